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
#include <cstring>
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

} // namespace nbvh

extern "C" {

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
