// TEST INFRASTRUCTURE: the oracle's own BVH builder, so that the CPU
// restatement of Tracer.comp (and bench.py's reference arm, which times it)
// builds its acceleration structure without loading the product library.
//
// The reference has no BVH (Assets/Tracer.comp:374-431 scans every primitive);
// the BVH is this project's extension, and the product builds it on the host
// (vk-renderer_gb300/csrc/bvh_build.cpp).  This file restates that builder's
// definition independently -- an explicit work list instead of recursion,
// index vectors instead of in-place partitions -- with the same decisions in
// the same IEEE double arithmetic, so that both produce the same nodes on every
// host (a CPU test compares them node for node):
//   * primitive box: the triangle's vertices (or the sphere's centre +- |r|);
//     centroid: (v0 + v1 + v2) / 3 in double (or the sphere's centre);
//   * a range of at most leaf_size primitives is a leaf;
//   * median split: order by centroid on the longest axis of the centroid box
//     (ties by primitive index), cut at the middle;
//   * binned SAH: `bins` equal-width bins of the centroid box per axis; the
//     plane k minimising N_left * A_left + N_right * A_right wins, first on a
//     strict improvement in the order axis 0..2, plane 0..bins-2; a range whose
//     centroids all coincide falls back to the median split; the partition
//     keeps each side's primitives in their previous order;
//   * a split that leaves one side empty becomes a cut at the middle;
//   * node box: the range's box padded by scale * 2^-14 + 1e-6 (scale = the
//     largest |coordinate| or extent), rounded outward to float;
//   * numbering: the root is node 0; an interior node's two children are
//     appended side by side when it is split, and the left subtree is split
//     completely before the right one.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle_api.h"

namespace {

struct OBox {
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL};
    double hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    void add_point(const double* p)
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    void add_box(const OBox& b)
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    double area() const
    {
        const double x = std::max(0.0, hi[0] - lo[0]), y = std::max(0.0, hi[1] - lo[1]),
                     z = std::max(0.0, hi[2] - lo[2]);
        return 2.0 * (x * y + y * z + z * x);
    }
};

struct ONode {
    float bmin[3];
    int32_t left_or_first;
    float bmax[3];
    int32_t count;
};
static_assert(sizeof(ONode) == 32, "node record is 32 bytes");

void padded_store(const OBox& b, ONode& n)
{
    double s = 0.0;
    for (int a = 0; a < 3; ++a) s = std::max({s, std::fabs(b.lo[a]), std::fabs(b.hi[a]), b.hi[a] - b.lo[a]});
    const double pad = s * 0x1.0p-14 + 1e-6;
    for (int a = 0; a < 3; ++a) {
        const double want_lo = b.lo[a] - pad, want_hi = b.hi[a] + pad;
        float flo = (float)want_lo, fhi = (float)want_hi;
        if ((double)flo > want_lo) flo = std::nextafter(flo, -HUGE_VALF);
        if ((double)fhi < want_hi) fhi = std::nextafter(fhi, HUGE_VALF);
        n.bmin[a] = flo;
        n.bmax[a] = fhi;
    }
}

struct OBuild {
    std::vector<OBox> box;
    std::vector<double> cen;  // 3 per primitive
    std::vector<uint32_t> order;
    std::vector<ONode> nodes;
    int kind = 0;
    uint32_t leaf = 4, bins = 16, depth = 0;

    OBox range_box(uint32_t b, uint32_t e, bool centroids) const
    {
        OBox r;
        for (uint32_t i = b; i < e; ++i) {
            if (centroids)
                r.add_point(&cen[3 * (size_t)order[i]]);
            else
                r.add_box(box[order[i]]);
        }
        return r;
    }

    uint32_t median_cut(uint32_t b, uint32_t e)
    {
        const OBox cb = range_box(b, e, true);
        int axis = 0;
        double widest = -1.0;
        for (int a = 0; a < 3; ++a)
            if (cb.hi[a] - cb.lo[a] > widest) {
                widest = cb.hi[a] - cb.lo[a];
                axis = a;
            }
        std::sort(order.begin() + b, order.begin() + e, [&](uint32_t x, uint32_t y) {
            const double u = cen[3 * (size_t)x + axis], v = cen[3 * (size_t)y + axis];
            return u < v || (u == v && x < y);
        });
        return b + (e - b) / 2;
    }

    static int64_t bin_of(double c, double lo, double scale, uint32_t nb)
    {
        int64_t k = (int64_t)((c - lo) * scale);
        return std::min<int64_t>(std::max<int64_t>(k, 0), (int64_t)nb - 1);
    }

    uint32_t sah_cut(uint32_t b, uint32_t e)
    {
        const OBox cb = range_box(b, e, true);
        int axis = -1;
        uint32_t plane = 0;
        double best = HUGE_VAL;
        for (int a = 0; a < 3; ++a) {
            const double ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.0)) continue;
            const double scale = (double)bins / ext;
            std::vector<OBox> bb(bins);
            std::vector<uint32_t> bn(bins, 0);
            for (uint32_t i = b; i < e; ++i) {
                const uint32_t p = order[i];
                const int64_t k = bin_of(cen[3 * (size_t)p + a], cb.lo[a], scale, bins);
                bb[k].add_box(box[p]);
                bn[k]++;
            }
            // right-hand sweep: area and count of bins k .. bins-1
            std::vector<double> ra(bins, 0.0);
            std::vector<uint32_t> rn(bins, 0);
            OBox r;
            uint32_t cnt = 0;
            for (uint32_t k = bins - 1; k >= 1; --k) {
                r.add_box(bb[k]);
                cnt += bn[k];
                ra[k] = r.area();
                rn[k] = cnt;
            }
            OBox l;
            uint32_t lc = 0;
            for (uint32_t k = 0; k + 1 < bins; ++k) {
                l.add_box(bb[k]);
                lc += bn[k];
                if (lc == 0 || rn[k + 1] == 0) continue;
                const double cost = (double)lc * l.area() + (double)rn[k + 1] * ra[k + 1];
                if (cost < best) {
                    best = cost;
                    axis = a;
                    plane = k;
                }
            }
        }
        if (axis < 0) return median_cut(b, e);
        const double scale = (double)bins / (cb.hi[axis] - cb.lo[axis]);
        std::vector<uint32_t> left, right;
        for (uint32_t i = b; i < e; ++i) {
            const uint32_t p = order[i];
            if (bin_of(cen[3 * (size_t)p + axis], cb.lo[axis], scale, bins) <= (int64_t)plane)
                left.push_back(p);
            else
                right.push_back(p);
        }
        std::copy(left.begin(), left.end(), order.begin() + b);
        std::copy(right.begin(), right.end(), order.begin() + b + left.size());
        return b + (uint32_t)left.size();
    }

    void run(uint32_t n)
    {
        struct Work {
            uint32_t node, b, e, level;
        };
        nodes.assign(1, ONode{});
        std::vector<Work> todo{{0, 0, n, 1}};
        while (!todo.empty()) {
            const Work w = todo.back();
            todo.pop_back();
            depth = std::max(depth, w.level);
            padded_store(range_box(w.b, w.e, false), nodes[w.node]);
            if (w.e - w.b <= leaf) {
                nodes[w.node].left_or_first = (int32_t)w.b;
                nodes[w.node].count = (int32_t)(w.e - w.b);
                continue;
            }
            uint32_t m = kind == 2 ? sah_cut(w.b, w.e) : median_cut(w.b, w.e);
            if (m <= w.b || m >= w.e) m = w.b + (w.e - w.b) / 2;
            const uint32_t c = (uint32_t)nodes.size();
            nodes.resize(nodes.size() + 2);
            nodes[w.node].left_or_first = (int32_t)c;
            nodes[w.node].count = 0;
            todo.push_back({c + 1, m, w.e, w.level + 1});  // right after left
            todo.push_back({c, w.b, m, w.level + 1});
        }
    }
};

}  // namespace

extern "C" int oracle_build_bvh(int kind, int prim_type, const void* prims, uint32_t n, uint32_t leaf_size,
                                uint32_t bins, void* nodes_out, uint32_t* num_nodes, uint32_t* prim_index_out,
                                uint32_t* depth_out)
{
    if (!prims || n == 0 || !nodes_out || !num_nodes || !prim_index_out) return -1;
    if ((kind != 1 && kind != 2) || (prim_type != 0 && prim_type != 1)) return -1;
    OBuild B;
    B.kind = kind;
    B.leaf = leaf_size ? leaf_size : (kind == 2 ? 4u : 2u);
    B.bins = bins ? bins : 16u;
    if (B.bins < 2 || B.bins > 256 || B.leaf > 64) return -1;
    B.box.resize(n);
    B.cen.resize(3 * (size_t)n);
    const float* f = static_cast<const float*>(prims);
    for (uint32_t i = 0; i < n; ++i) {
        if (prim_type == 0) {  // 48 B triangle: v0 @0, v1 @16, v2 @32
            const float* t = f + 12 * (size_t)i;
            for (int k = 0; k < 3; ++k) {
                const double v[3] = {t[4 * k], t[4 * k + 1], t[4 * k + 2]};
                B.box[i].add_point(v);
            }
            for (int a = 0; a < 3; ++a)
                B.cen[3 * (size_t)i + a] = ((double)t[a] + (double)t[4 + a] + (double)t[8 + a]) / 3.0;
        } else {  // 64 B sphere: centre @48, radius @60
            const float* s = f + 16 * (size_t)i;
            const double r = std::fabs((double)s[15]);
            for (int a = 0; a < 3; ++a) {
                B.box[i].lo[a] = (double)s[12 + a] - r;
                B.box[i].hi[a] = (double)s[12 + a] + r;
                B.cen[3 * (size_t)i + a] = s[12 + a];
            }
        }
    }
    B.order.resize(n);
    for (uint32_t i = 0; i < n; ++i) B.order[i] = i;
    B.run(n);
    std::memcpy(nodes_out, B.nodes.data(), B.nodes.size() * sizeof(ONode));
    std::memcpy(prim_index_out, B.order.data(), (size_t)n * sizeof(uint32_t));
    *num_nodes = (uint32_t)B.nodes.size();
    if (depth_out) *depth_out = B.depth;
    return 0;
}
