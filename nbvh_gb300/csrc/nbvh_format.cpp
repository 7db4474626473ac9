// nbvh_format.cpp -- the reference's .nbvh neural-cut file.
//
// The reference saves and loads its neural BVH (NeuralBVHRenderer::save_neural_bvh /
// load_neural_bvh, src/cuda/neural/neural_bvh_renderer_accel.cpp:170-254) through the madmann91/bvh
// v2 serializer, a submodule whose pinned version is not in the reference tree. The layout below
// is the one the reference's shipped cut file shows (all little-endian):
//
//   u64 n                  number of nodes
//   u64 1
//   n x 40-byte records    f32 min.x, max.x, min.y, max.y, min.z, max.z, u64 first_id, u64 prim_count
//   u64 0                  the serializer's single primitive id
//
// first_id is the left child of an interior node (prim_count 0; the right child follows it) and
// 0xFFFFFFFF (NO_NEURAL_CHILD) for a leaf; a leaf's prim_count is 1 (final leaf) or LoD + 2.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "nbvh_internal.h"

using namespace nbvh;

namespace {

constexpr uint64_t kRecordBytes = 40;

void put_u64(std::vector<unsigned char> &b, uint64_t v)
{
    for (int k = 0; k < 8; k++)
        b.push_back((unsigned char)(v >> (8 * k)));
}

void put_f32(std::vector<unsigned char> &b, float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    for (int k = 0; k < 4; k++)
        b.push_back((unsigned char)(u >> (8 * k)));
}

uint64_t get_u64(const unsigned char *p)
{
    uint64_t v = 0;
    for (int k = 7; k >= 0; k--)
        v = (v << 8) | p[k];
    return v;
}

float get_f32(const unsigned char *p)
{
    uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

} // namespace

namespace nbvh {

// Structural checks of a neural cut: every interior node's two children exist and are not the
// node itself, leaves carry NO_NEURAL_CHILD and a prim_count of 1..8, boxes are ordered, and the
// tree below the root reaches every node once.
bool validate_cut(const std::vector<BVHNode> &nodes, std::string &err)
{
    const size_t n = nodes.size();
    if (n == 0 || n > (1u << 30)) {
        err = "node count out of range";
        return false;
    }
    for (size_t i = 0; i < n; i++) {
        const BVHNode &nd = nodes[i];
        for (int k = 0; k < 3; k++)
            if (!(nd.min[k] <= nd.max[k])) {
                err = "node " + std::to_string(i) + ": box min above max";
                return false;
            }
        if (nd.prim_count == 0u) {
            const uint64_t c = nd.left_or_prim_offset;
            if (c + 1u >= n || c == i || c + 1u == i) {
                err = "node " + std::to_string(i) + ": child index out of range";
                return false;
            }
        } else if (nd.prim_count > 8u || nd.left_or_prim_offset != kNoNeuralChild) {
            err = "node " + std::to_string(i) + ": malformed leaf";
            return false;
        }
    }
    std::vector<uint8_t> seen(n, 0u);
    std::vector<uint32_t> stack{0u};
    size_t visited = 0;
    while (!stack.empty()) {
        const uint32_t i = stack.back();
        stack.pop_back();
        if (seen[i]) {
            err = "node " + std::to_string(i) + " reached twice";
            return false;
        }
        seen[i] = 1u;
        visited++;
        if (nodes[i].prim_count == 0u) {
            stack.push_back(nodes[i].left_or_prim_offset);
            stack.push_back(nodes[i].left_or_prim_offset + 1u);
        }
    }
    if (visited != n) {
        err = "nodes unreachable from the root";
        return false;
    }
    return true;
}

bool read_nbvh(const std::string &path, std::vector<BVHNode> &nodes, std::string &err)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<unsigned char> buf;
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0)
        buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    if (buf.size() < 24) {
        err = "file too short";
        return false;
    }
    const uint64_t n = get_u64(buf.data());
    if (n == 0 || n > (1ull << 30) || buf.size() != 16u + n * kRecordBytes + 8u) {
        err = "size does not match the node count";
        return false;
    }
    if (get_u64(buf.data() + 8) != 1u || get_u64(buf.data() + buf.size() - 8) != 0u) {
        err = "unexpected header or trailer";
        return false;
    }
    nodes.resize((size_t)n);
    for (uint64_t i = 0; i < n; i++) {
        const unsigned char *r = buf.data() + 16 + i * kRecordBytes;
        BVHNode &nd = nodes[(size_t)i];
        for (int k = 0; k < 3; k++) {
            nd.min[k] = get_f32(r + 8 * k);
            nd.max[k] = get_f32(r + 8 * k + 4);
        }
        const uint64_t first = get_u64(r + 24), count = get_u64(r + 32);
        if (first > 0xFFFFFFFFull || count > 0xFFFFFFFFull) {
            err = "node " + std::to_string(i) + ": index out of range";
            return false;
        }
        nd.left_or_prim_offset = (uint32_t)first;
        nd.prim_count = (uint32_t)count;
    }
    return validate_cut(nodes, err);
}

bool write_nbvh(const std::string &path, const std::vector<BVHNode> &nodes, std::string &err)
{
    std::vector<unsigned char> buf;
    buf.reserve(24 + nodes.size() * kRecordBytes);
    put_u64(buf, nodes.size());
    put_u64(buf, 1u);
    for (const BVHNode &nd : nodes) {
        for (int k = 0; k < 3; k++) {
            put_f32(buf, nd.min[k]);
            put_f32(buf, nd.max[k]);
        }
        put_u64(buf, nd.left_or_prim_offset);
        put_u64(buf, nd.prim_count);
    }
    put_u64(buf, 0u);
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "cannot create " + path;
        return false;
    }
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    ok ? (void)0 : (void)(err = "write failed");
    return (std::fclose(f) == 0) && ok;
}

// ---------------------------------------------------------------------------------------------
// tcnn trainer weights as the reference saves them (NeuralBVHRenderer::save_network_model /
// load_network_model, src/cuda/neural/neural_bvh_renderer_init.cu:385-404): the JSON object of
// trainer->serialize(false) written as text, {"n_params": N, "params_type": "float" | "__half",
// "params_binary": B}, where B is a JSON binary value, which nlohmann's text form writes as
// {"bytes": [b0, b1, ...], "subtype": null}. tiny-cuda-nn is an empty submodule of the reference
// tree; this follows the fields its trainer serializes. The element size is taken from the byte
// count (4 N: FP32, 2 N: FP16), params_type only has to agree with it.
// ---------------------------------------------------------------------------------------------

namespace {

struct JsonScan {
    const std::string &t;
    size_t i = 0;
    explicit JsonScan(const std::string &text) : t(text) {}
    void ws()
    {
        while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t'))
            i++;
    }
    bool lit(char c)
    {
        ws();
        if (i < t.size() && t[i] == c) {
            i++;
            return true;
        }
        return false;
    }
    bool str(std::string &out)
    {
        ws();
        if (i >= t.size() || t[i] != '"')
            return false;
        out.clear();
        for (i++; i < t.size() && t[i] != '"'; i++) {
            if (t[i] == '\\') { // escapes do not occur in the keys and values read here
                if (++i >= t.size())
                    return false;
            }
            out.push_back(t[i]);
        }
        return i++ < t.size();
    }
    bool uint(uint64_t &v)
    {
        ws();
        if (i >= t.size() || t[i] < '0' || t[i] > '9')
            return false;
        v = 0;
        while (i < t.size() && t[i] >= '0' && t[i] <= '9') {
            if (v > (UINT64_MAX - 9u) / 10u)
                return false;
            v = v * 10u + (uint64_t)(t[i++] - '0');
        }
        return true;
    }
    // skips any JSON value (objects and arrays by nesting; strings with escapes)
    bool skip()
    {
        ws();
        if (i >= t.size())
            return false;
        if (t[i] == '"') {
            std::string tmp;
            return str(tmp);
        }
        if (t[i] == '{' || t[i] == '[') {
            int depth = 0;
            bool in_str = false;
            for (; i < t.size(); i++) {
                const char c = t[i];
                if (in_str) {
                    if (c == '\\')
                        i++;
                    else if (c == '"')
                        in_str = false;
                } else if (c == '"') {
                    in_str = true;
                } else if (c == '{' || c == '[') {
                    depth++;
                } else if (c == '}' || c == ']') {
                    if (--depth == 0) {
                        i++;
                        return true;
                    }
                }
            }
            return false;
        }
        while (i < t.size() && t[i] != ',' && t[i] != '}' && t[i] != ']')
            i++;
        return true;
    }
    // [b0, b1, ...] of values 0..255
    bool byte_array(std::vector<unsigned char> &out)
    {
        if (!lit('['))
            return false;
        out.clear();
        if (lit(']'))
            return true;
        for (;;) {
            uint64_t v;
            if (!uint(v) || v > 255u)
                return false;
            out.push_back((unsigned char)v);
            if (lit(']'))
                return true;
            if (!lit(','))
                return false;
        }
    }
};

float half_bits_to_float(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h >> 15) << 31, ex = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
    uint32_t u;
    if (ex == 0u) {
        if (man == 0u) {
            u = sign;
        } else { // subnormal: normalise
            int e = -1;
            uint32_t m = man;
            do {
                e++;
                m <<= 1;
            } while ((m & 0x400u) == 0u);
            u = sign | ((uint32_t)(127 - 15 - e) << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (ex == 0x1Fu) {
        u = sign | 0x7F800000u | (man << 13);
    } else {
        u = sign | ((ex - 15u + 127u) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

} // namespace

bool read_tcnn_params(const char *path, std::vector<float> &params, std::string &err)
{
    std::FILE *f = std::fopen(path, "rb");
    if (!f) {
        err = "cannot open";
        return false;
    }
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0)
        text.append(buf, got);
    std::fclose(f);
    JsonScan js(text);
    if (!js.lit('{')) {
        err = "not a JSON object";
        return false;
    }
    uint64_t n = 0;
    bool have_n = false;
    std::string type;
    std::vector<unsigned char> bytes;
    bool have_bytes = false;
    if (!js.lit('}')) {
        for (;;) {
            std::string key;
            if (!js.str(key) || !js.lit(':')) {
                err = "malformed object";
                return false;
            }
            if (key == "n_params") {
                have_n = js.uint(n);
            } else if (key == "params_type") {
                if (!js.str(type)) {
                    err = "params_type is not a string";
                    return false;
                }
            } else if (key == "params_binary") {
                // {"bytes": [...], "subtype": ...} (text form of a binary value) or a bare array
                js.ws();
                if (js.i < text.size() && text[js.i] == '[') {
                    have_bytes = js.byte_array(bytes);
                } else if (js.lit('{')) {
                    for (;;) {
                        std::string k2;
                        if (!js.str(k2) || !js.lit(':')) {
                            err = "malformed params_binary";
                            return false;
                        }
                        if (k2 == "bytes")
                            have_bytes = js.byte_array(bytes);
                        else if (!js.skip())
                            break;
                        if (js.lit('}'))
                            break;
                        if (!js.lit(',')) {
                            err = "malformed params_binary";
                            return false;
                        }
                    }
                }
                if (!have_bytes) {
                    err = "params_binary has no byte array";
                    return false;
                }
            } else if (!js.skip()) {
                err = "malformed value of " + key;
                return false;
            }
            if (js.lit('}'))
                break;
            if (!js.lit(',')) {
                err = "malformed object";
                return false;
            }
        }
    }
    if (!have_n || !have_bytes) {
        err = "n_params or params_binary missing";
        return false;
    }
    if (n == 0 || n > (1ull << 31)) {
        err = "bad n_params";
        return false;
    }
    const bool f32 = bytes.size() == 4u * n, f16 = bytes.size() == 2u * n;
    if (!f32 && !f16) {
        err = "params_binary holds " + std::to_string(bytes.size()) + " bytes for " + std::to_string(n) + " parameters";
        return false;
    }
    if (!type.empty() && ((f32 && type != "float") || (f16 && type != "__half"))) {
        err = "params_type " + type + " does not match the byte count";
        return false;
    }
    params.resize(n);
    for (uint64_t k = 0; k < n; k++) {
        if (f32) {
            const unsigned char *p = bytes.data() + 4u * k;
            const uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
            std::memcpy(&params[k], &u, 4);
        } else {
            const unsigned char *p = bytes.data() + 2u * k;
            params[k] = half_bits_to_float((uint16_t)(p[0] | (p[1] << 8)));
        }
    }
    return true;
}

bool write_tcnn_params(const char *path, const float *params, uint64_t n, std::string &err)
{
    std::FILE *f = std::fopen(path, "wb");
    if (!f) {
        err = "cannot open";
        return false;
    }
    std::string out;
    out.reserve(64u + 16u * n);
    out += "{\"n_params\":" + std::to_string(n) + ",\"params_binary\":{\"bytes\":[";
    for (uint64_t k = 0; k < n; k++) {
        uint32_t u;
        std::memcpy(&u, &params[k], 4);
        for (int b = 0; b < 4; b++) {
            if (k || b)
                out.push_back(',');
            out += std::to_string((u >> (8 * b)) & 0xFFu);
        }
    }
    out += "],\"subtype\":null},\"params_type\":\"float\"}";
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    if (!ok)
        err = "write failed";
    return (std::fclose(f) == 0) && ok;
}

} // namespace nbvh

extern "C" {

nbvh_status nbvh_read_tcnn_params_host(const char *path, float *h_params, uint64_t capacity, uint64_t *n_params)
{
    if (!path || !n_params)
        return NBVH_EINVAL;
    std::vector<float> p;
    std::string err;
    if (!read_tcnn_params(path, p, err))
        return NBVH_EIO;
    *n_params = p.size();
    if (h_params) {
        if (capacity < p.size())
            return NBVH_EINVAL;
        std::memcpy(h_params, p.data(), p.size() * sizeof(float));
    }
    return NBVH_OK;
}

nbvh_status nbvh_write_tcnn_params_host(const char *path, const float *h_params, uint64_t n_params)
{
    if (!path || !h_params || n_params == 0)
        return NBVH_EINVAL;
    std::string err;
    return write_tcnn_params(path, h_params, n_params, err) ? NBVH_OK : NBVH_EIO;
}

nbvh_status nbvh_read_nbvh_host(const char *path, uint32_t *h_nodes, uint32_t *n_nodes)
{
    if (!path || !n_nodes)
        return NBVH_EINVAL;
    std::vector<BVHNode> nodes;
    std::string err;
    if (!read_nbvh(path, nodes, err))
        return NBVH_EIO;
    if (h_nodes) {
        if (*n_nodes < nodes.size())
            return NBVH_EINVAL;
        std::memcpy(h_nodes, nodes.data(), nodes.size() * sizeof(BVHNode));
    }
    *n_nodes = (uint32_t)nodes.size();
    return NBVH_OK;
}

nbvh_status nbvh_write_nbvh_host(const char *path, const uint32_t *h_nodes, uint32_t n_nodes)
{
    if (!path || !h_nodes || n_nodes == 0)
        return NBVH_EINVAL;
    std::vector<BVHNode> nodes(n_nodes);
    std::memcpy(nodes.data(), h_nodes, (size_t)n_nodes * sizeof(BVHNode));
    std::string err;
    if (!validate_cut(nodes, err))
        return NBVH_EINVAL;
    return write_nbvh(path, nodes, err) ? NBVH_OK : NBVH_EIO;
}

} // extern "C"
