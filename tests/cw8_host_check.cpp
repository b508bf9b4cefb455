// Host check of the compressed 8-wide BVH builder (vk-renderer_gb300/csrc/
// bvh_cw8.cpp), compiled by tests/test_cw8_host.py together with the binary
// builder: structural invariants of the nodes (every index the device kernel
// will read is in range, every primitive referenced once, every quantised box
// contains its binary child's box) and a host emulation of the device
// traversal (tracer_cw8.cuh: the same float slab test, node groups and
// visiting order) whose closest hits must equal a brute-force scan's.
//
// Usage: cw8_host_check <n_triangles> <extent> <sigma> <leaf> <rays> <seed>
// Prints "ok nodes=<n> depth=<d> hits=<h>", "refused" (leaves beyond the 8-wide
// limit), or "FAIL ..." (exit 1).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bvh_cw8.h"
#include "tracer_abi.h"

using vkt::Cw8Node;

namespace {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (double)(next() >> 11) * 0x1.0p-53; }
    double normal()
    {
        const double u = std::max(uni(), 1e-300), v = uni();
        return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
    }
};

[[noreturn]] void fail(const char* what, long a = 0, long b = 0)
{
    std::printf("FAIL %s %ld %ld\n", what, a, b);
    std::exit(1);
}

// Moller-Trumbore, one-sided, as the device's tri_intersect (float, no fma)
float tri_t(const float o[3], const float d[3], const float v0[3], const float e1[3], const float e2[3])
{
    const float p[3] = {d[1] * e2[2] - e2[1] * d[2], d[2] * e2[0] - e2[2] * d[0], d[0] * e2[1] - e2[0] * d[1]};
    const float det = (e1[0] * p[0] + e1[1] * p[1]) + e1[2] * p[2];
    if (det < 1e-3f) return -1.0f;
    const float inv = 1.0f / det;
    const float tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
    const float u = ((tv[0] * p[0] + tv[1] * p[1]) + tv[2] * p[2]) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const float q[3] = {tv[1] * e1[2] - e1[1] * tv[2], tv[2] * e1[0] - e1[2] * tv[0], tv[0] * e1[1] - e1[0] * tv[1]};
    const float v = ((d[0] * q[0] + d[1] * q[1]) + d[2] * q[2]) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    return ((e2[0] * q[0] + e2[1] * q[1]) + e2[2] * q[2]) * inv;
}

struct Best {
    float t;
    uint32_t id;
};

void accept(Best& b, float t, uint32_t id)
{
    if (t > 1e-3f && (t < b.t || (t == b.t && id < b.id))) {
        b.t = t;
        b.id = id;
    }
}

float safe_inv(float d) { return 1.0f / ((std::fabs(d) > 1e-30f) ? d : std::copysign(1e-30f, d)); }
uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }
float f_of(uint32_t w)
{
    float f;
    std::memcpy(&f, &w, 4);
    return f;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 7) return 2;
    const uint32_t n = (uint32_t)std::atoi(argv[1]);
    const double extent = std::atof(argv[2]), sigma = std::atof(argv[3]);
    const uint32_t leaf = (uint32_t)std::atoi(argv[4]), nrays = (uint32_t)std::atoi(argv[5]);
    Rng g{(uint64_t)std::atoll(argv[6])};
    std::vector<tracer_triangle> tris(n);
    for (auto& t : tris) {
        double c[3];
        for (double& x : c) x = extent * (2.0 * g.uni() - 1.0);
        float* v[3] = {t.v0, t.v1, t.v2};
        for (float* p : v)
            for (int a = 0; a < 3; ++a) p[a] = (float)(c[a] + sigma * g.normal());
        t.material = 0;
    }
    std::vector<tracer_bvh_node> nodes(2 * (size_t)n);
    std::vector<uint32_t> idx(n);
    uint32_t nn = 0, bdepth = 0;
    if (tracer_build_bvh(TRACER_BVH_SAH, TRACER_PRIM_TRIANGLE, tris.data(), n, leaf, 16, nodes.data(), &nn, idx.data(),
                         &bdepth) != TRACER_OK)
        fail("binary build");
    nodes.resize(nn);
    std::vector<Cw8Node> w;
    std::vector<uint32_t> order;
    uint32_t depth = 0;
    if (!vkt::build_cw8(nodes.data(), nn, w, order, &depth)) {
        // refused: only for leaves beyond kCw8MaxLeafPrims
        if (leaf > vkt::kCw8MaxLeafPrims) {
            std::printf("refused\n");
            return 0;
        }
        fail("build_cw8 refused");
    }
    if (leaf > vkt::kCw8MaxLeafPrims) {
        bool big = false;
        for (const auto& nd : nodes) big = big || nd.count > (int32_t)vkt::kCw8MaxLeafPrims;
        if (big) fail("accepted a leaf beyond the limit");
    }
    if (depth > bdepth) fail("8-wide deeper than binary", depth, bdepth);
    // structure: indices in range, every primitive once
    if (order.size() != n) fail("order size", (long)order.size(), n);
    std::vector<int> seen(n, 0);
    for (uint32_t s : order) {
        if (s >= n) fail("order slot", s);
        seen[s]++;
    }
    for (uint32_t i = 0; i < n; ++i)
        if (seen[i] != 1) fail("slot count", i, seen[i]);
    for (size_t i = 0; i < w.size(); ++i) {
        const uint32_t* x = w[i].w;
        const uint32_t imask = x[3] >> 24;
        int ni = 0;
        uint32_t used = 0;
        for (int k = 0; k < 8; ++k) {
            const uint32_t xm = byte_of(x[6 + k / 4], k % 4), bits = byte_of(x[20 + k / 4], k % 4),
                           pos = byte_of(x[22 + k / 4], k % 4);
            const bool inner = (imask >> k) & 1u;
            if (xm != (inner ? 7u : 0u)) fail("octant mask", (long)i, k);
            if (inner) {
                ++ni;
                if (bits != 1u || pos != 24u + (uint32_t)k) fail("interior bits", (long)i, k);
            } else if (bits != 0u) {
                const uint32_t c = (uint32_t)__builtin_popcount(bits);
                if (bits != (1u << c) - 1u || c > vkt::kCw8MaxLeafPrims || pos + c > 24u) fail("leaf bits", (long)i, k);
                if (used & (bits << pos)) fail("overlapping leaves", (long)i, k);
                used |= bits << pos;
                if ((size_t)x[5] + pos + c > n) fail("prim range", (long)i, k);
            } else if (pos != 0u) {
                fail("empty slot", (long)i, k);
            }
        }
        if (ni && (size_t)x[4] + ni > w.size()) fail("child range", (long)i, x[4]);
    }
    // traversal emulation against a brute-force scan
    std::vector<float> v0(3 * (size_t)n), e1(3 * (size_t)n), e2(3 * (size_t)n);
    std::vector<uint32_t> orig(n);
    for (uint32_t k = 0; k < n; ++k) {
        const tracer_triangle& t = tris[idx[order[k]]];
        for (int a = 0; a < 3; ++a) {
            v0[3 * k + a] = t.v0[a];
            e1[3 * k + a] = t.v1[a] - t.v0[a];
            e2[3 * k + a] = t.v2[a] - t.v0[a];
        }
        orig[k] = idx[order[k]];
    }
    uint32_t hits = 0;
    std::vector<uint64_t> stack;
    for (uint32_t r = 0; r < nrays; ++r) {
        float o[3], d[3];
        for (int a = 0; a < 3; ++a) o[a] = (float)(1.3 * extent * (2.0 * g.uni() - 1.0));
        for (int a = 0; a < 3; ++a) d[a] = (float)g.normal();
        if (r % 17 == 0) d[r % 3] = 0.0f;  // axis-parallel directions too
        const float tmax = (r % 5 == 0) ? 3.0f : 3000.0f;
        Best brute{tmax, 0};
        for (uint32_t k = 0; k < n; ++k) accept(brute, tri_t(o, d, &v0[3 * k], &e1[3 * k], &e2[3 * k]), orig[k]);
        const float ix = safe_inv(d[0]), iy = safe_inv(d[1]), iz = safe_inv(d[2]);
        const float nx = -(o[0] * ix), ny = -(o[1] * iy), nz = -(o[2] * iz);
        const uint32_t oct7 = ((ix < 0) | (iy < 0) << 1 | (iz < 0) << 2) ^ 7u;
        Best b{tmax, 0};
        uint64_t G = (uint64_t)((1u << (24 + (0u ^ oct7))) | 1u) << 32;  // (base 0, root bit | imask 1)
        stack.clear();
        for (;;) {
            if (((G >> 32) & 0xFF000000u) == 0) {
                if (stack.empty()) break;
                G = stack.back();
                stack.pop_back();
            }
            uint32_t base = (uint32_t)G, gy = (uint32_t)(G >> 32);
            const int bit = 31 - __builtin_clz(gy);
            const uint32_t slot = (uint32_t)(bit - 24) ^ oct7;
            gy &= ~(1u << bit);
            const uint32_t ci = base + __builtin_popcount(gy & ((1u << slot) - 1u) & 0xFFu);
            if (gy & 0xFF000000u) stack.push_back((uint64_t)gy << 32 | base);
            if (ci >= w.size()) fail("visit index", ci);
            const uint32_t* x = w[ci].w;
            const float sx = f_of((x[3] & 0xFFu) << 23), sy = f_of(((x[3] >> 8) & 0xFFu) << 23),
                        sz = f_of(((x[3] >> 16) & 0xFFu) << 23);
            const float ax = sx * ix, ay = sy * iy, az = sz * iz;
            const float bx = std::fma(f_of(x[0]), ix, nx), by = std::fma(f_of(x[1]), iy, ny),
                        bz = std::fma(f_of(x[2]), iz, nz);
            uint32_t mask = 0;
            for (int k = 0; k < 8; ++k) {
                const int h = k / 4, kk = k % 4;
                const float lx = (float)byte_of(x[8 + h], kk), ly = (float)byte_of(x[10 + h], kk),
                            lz = (float)byte_of(x[12 + h], kk), hx = (float)byte_of(x[14 + h], kk),
                            hy = (float)byte_of(x[16 + h], kk), hz = (float)byte_of(x[18 + h], kk);
                const float tnx = std::fma(ix < 0 ? hx : lx, ax, bx), tfx = std::fma(ix < 0 ? lx : hx, ax, bx);
                const float tny = std::fma(iy < 0 ? hy : ly, ay, by), tfy = std::fma(iy < 0 ? ly : hy, ay, by);
                const float tnz = std::fma(iz < 0 ? hz : lz, az, bz), tfz = std::fma(iz < 0 ? lz : hz, az, bz);
                const float tmn = std::fmax(std::fmax(std::fmax(tnx, tny), tnz), 0.0f);
                const float tmx = std::fmin(std::fmin(std::fmin(tfx, tfy), tfz), b.t);
                const uint32_t bits = byte_of(x[20 + h], kk), pos = byte_of(x[22 + h], kk) ^ (oct7 & byte_of(x[6 + h], kk));
                if (tmn <= tmx * (1.0f + 0x1.0p-20f)) mask |= bits << pos;
            }
            for (uint32_t p = mask & 0x00FFFFFFu; p; p &= p - 1) {
                const uint32_t k = x[5] + __builtin_ctz(p);
                accept(b, tri_t(o, d, &v0[3 * k], &e1[3 * k], &e2[3 * k]), orig[k]);
            }
            G = (uint64_t)((mask & 0xFF000000u) | (x[3] >> 24)) << 32 | x[4];
        }
        if (b.t != brute.t || b.id != brute.id) fail("closest hit differs", r, (long)b.id);
        if (brute.t < tmax) ++hits;
    }
    std::printf("ok nodes=%zu depth=%u binary_depth=%u hits=%u\n", w.size(), depth, bdepth, hits);
    return 0;
}
