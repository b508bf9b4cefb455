// Host BVH builders (median split and binned SAH) and validator.
//
// The reference traces by a linear scan over every primitive
// (Assets/Tracer.comp:378-428); it has no acceleration structure.  The BVH is
// this project's extension and is built here, on the host, deterministically:
// every decision uses IEEE double arithmetic with a total order (ties broken
// by primitive index), so x86 and aarch64 hosts produce identical trees.
//
// Layout: tracer_bvh_node (32 B).  Children of an interior node are stored
// side by side (left, left + 1) so one 64-byte read fetches both; node 0 is
// the root.  Node boxes are padded outward by a small relative margin so that
// the float slab test in traversal never culls a box whose primitive the
// Moller-Trumbore test would report as hit.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "tracer_abi.h"

namespace {

struct Box {
    double lo[3], hi[3];
    void reset()
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = HUGE_VAL;
            hi[a] = -HUGE_VAL;
        }
    }
    void grow(const Box& b)
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void grow_pt(const double p[3])
    {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    double area() const
    {
        double e[3];
        for (int a = 0; a < 3; ++a) e[a] = std::max(0.0, hi[a] - lo[a]);
        return 2.0 * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
    }
};

struct Prim {
    Box box;
    double c[3];  // centroid
};

std::vector<Prim> make_prims(int prim_type, const void* prims, uint32_t n)
{
    std::vector<Prim> out(n);
    for (uint32_t i = 0; i < n; ++i) {
        Prim& p = out[i];
        p.box.reset();
        if (prim_type == TRACER_PRIM_TRIANGLE) {
            const tracer_triangle& t = static_cast<const tracer_triangle*>(prims)[i];
            const float* v[3] = {t.v0, t.v1, t.v2};
            for (int k = 0; k < 3; ++k) {
                double q[3] = {v[k][0], v[k][1], v[k][2]};
                p.box.grow_pt(q);
            }
            for (int a = 0; a < 3; ++a) p.c[a] = ((double)t.v0[a] + (double)t.v1[a] + (double)t.v2[a]) / 3.0;
        } else {
            const tracer_sphere& s = static_cast<const tracer_sphere*>(prims)[i];
            double r = std::fabs((double)s.r);
            for (int a = 0; a < 3; ++a) {
                p.box.lo[a] = (double)s.P[a] - r;
                p.box.hi[a] = (double)s.P[a] + r;
                p.c[a] = s.P[a];
            }
        }
    }
    return out;
}

// Outward padding of a node box, then rounding to float outward.
void store_box(const Box& b, tracer_bvh_node& nd)
{
    double scale = 0.0;
    for (int a = 0; a < 3; ++a) {
        scale = std::max(scale, std::fabs(b.lo[a]));
        scale = std::max(scale, std::fabs(b.hi[a]));
        scale = std::max(scale, b.hi[a] - b.lo[a]);
    }
    const double pad = scale * 0x1.0p-14 + 1e-6;
    for (int a = 0; a < 3; ++a) {
        float lo = (float)(b.lo[a] - pad);
        float hi = (float)(b.hi[a] + pad);
        if ((double)lo > b.lo[a] - pad) lo = std::nextafter(lo, -HUGE_VALF);
        if ((double)hi < b.hi[a] + pad) hi = std::nextafter(hi, HUGE_VALF);
        nd.bmin[a] = lo;
        nd.bmax[a] = hi;
    }
}

struct Builder {
    const std::vector<Prim>& prims;
    int kind;
    uint32_t leaf_size, bins;
    std::vector<uint32_t> idx;  // primitive order; leaves are ranges of it
    std::vector<tracer_bvh_node> nodes;
    uint32_t depth = 0;

    Box bounds(uint32_t b, uint32_t e) const
    {
        Box bx;
        bx.reset();
        for (uint32_t i = b; i < e; ++i) bx.grow(prims[idx[i]].box);
        return bx;
    }
    Box cbounds(uint32_t b, uint32_t e) const
    {
        Box bx;
        bx.reset();
        for (uint32_t i = b; i < e; ++i) bx.grow_pt(prims[idx[i]].c);
        return bx;
    }

    // Median split: sort by centroid on the longest centroid axis (ties by
    // index) and cut at the middle.
    uint32_t split_median(uint32_t b, uint32_t e)
    {
        Box cb = cbounds(b, e);
        int axis = 0;
        double best = -1.0;
        for (int a = 0; a < 3; ++a) {
            double ext = cb.hi[a] - cb.lo[a];
            if (ext > best) {
                best = ext;
                axis = a;
            }
        }
        std::sort(idx.begin() + b, idx.begin() + e, [&](uint32_t x, uint32_t y) {
            double cx = prims[x].c[axis], cy = prims[y].c[axis];
            return cx < cy || (cx == cy && x < y);
        });
        return b + (e - b) / 2;
    }

    // Binned SAH: `bins` equal bins of the centroid box per axis; the split
    // plane with the least  N_left*A_left + N_right*A_right  wins (ties: lower
    // axis, then lower plane).  Falls back to the median split when all
    // centroids coincide.
    uint32_t split_sah(uint32_t b, uint32_t e)
    {
        Box cb = cbounds(b, e);
        int best_axis = -1;
        uint32_t best_plane = 0;
        double best_cost = HUGE_VAL;
        std::vector<Box> bb(bins);
        std::vector<uint32_t> bc(bins);
        std::vector<double> rarea(bins);
        std::vector<uint32_t> rcount(bins);
        for (int a = 0; a < 3; ++a) {
            double ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.0)) continue;
            double scale = (double)bins / ext;
            for (uint32_t k = 0; k < bins; ++k) {
                bb[k].reset();
                bc[k] = 0;
            }
            for (uint32_t i = b; i < e; ++i) {
                const Prim& p = prims[idx[i]];
                int64_t k = (int64_t)((p.c[a] - cb.lo[a]) * scale);
                k = std::min<int64_t>(std::max<int64_t>(k, 0), bins - 1);
                bb[k].grow(p.box);
                bc[k]++;
            }
            Box acc;
            acc.reset();
            uint32_t cnt = 0;
            for (uint32_t k = bins - 1; k >= 1; --k) {
                acc.grow(bb[k]);
                cnt += bc[k];
                rarea[k] = acc.area();
                rcount[k] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (uint32_t k = 0; k + 1 < bins; ++k) {
                acc.grow(bb[k]);
                cnt += bc[k];
                uint32_t rc = rcount[k + 1];
                if (cnt == 0 || rc == 0) continue;
                double cost = (double)cnt * acc.area() + (double)rc * rarea[k + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_plane = k;
                }
            }
        }
        if (best_axis < 0) return split_median(b, e);
        const int a = best_axis;
        const double scale = (double)bins / (cb.hi[a] - cb.lo[a]);
        auto it = std::stable_partition(idx.begin() + b, idx.begin() + e, [&](uint32_t x) {
            int64_t k = (int64_t)((prims[x].c[a] - cb.lo[a]) * scale);
            k = std::min<int64_t>(std::max<int64_t>(k, 0), bins - 1);
            return k <= (int64_t)best_plane;
        });
        return (uint32_t)(it - idx.begin());
    }

    void build(uint32_t node, uint32_t b, uint32_t e, uint32_t level)
    {
        depth = std::max(depth, level);
        store_box(bounds(b, e), nodes[node]);
        if (e - b <= leaf_size) {
            nodes[node].left_or_first = (int32_t)b;
            nodes[node].count = (int32_t)(e - b);
            return;
        }
        uint32_t m = kind == TRACER_BVH_SAH ? split_sah(b, e) : split_median(b, e);
        if (m <= b || m >= e) m = b + (e - b) / 2;
        uint32_t l = (uint32_t)nodes.size();
        nodes.emplace_back();
        nodes.emplace_back();
        nodes[node].left_or_first = (int32_t)l;
        nodes[node].count = 0;
        build(l, b, m, level + 1);
        build(l + 1, m, e, level + 1);
    }
};

}  // namespace

extern "C" int tracer_build_bvh(int kind, int prim_type, const void* prims, uint32_t n, uint32_t leaf_size,
                                uint32_t sah_bins, tracer_bvh_node* nodes_out, uint32_t* num_nodes_out,
                                uint32_t* prim_index_out, uint32_t* depth_out)
{
    if (!prims || n == 0 || !nodes_out || !num_nodes_out || !prim_index_out) return TRACER_ERR_INVALID_ARG;
    if (kind != TRACER_BVH_MEDIAN && kind != TRACER_BVH_SAH) return TRACER_ERR_INVALID_ARG;
    if (prim_type != TRACER_PRIM_TRIANGLE && prim_type != TRACER_PRIM_SPHERE) return TRACER_ERR_INVALID_ARG;
    if (leaf_size == 0) leaf_size = kind == TRACER_BVH_SAH ? 4 : 2;
    if (sah_bins == 0) sah_bins = 16;
    if (sah_bins < 2 || sah_bins > 256 || leaf_size > 64) return TRACER_ERR_INVALID_ARG;
    std::vector<Prim> p = make_prims(prim_type, prims, n);
    Builder bld{p, kind, leaf_size, sah_bins, {}, {}, 0};
    bld.idx.resize(n);
    for (uint32_t i = 0; i < n; ++i) bld.idx[i] = i;
    bld.nodes.reserve(2 * (size_t)n);
    bld.nodes.emplace_back();
    bld.build(0, 0, n, 1);
    std::memcpy(nodes_out, bld.nodes.data(), bld.nodes.size() * sizeof(tracer_bvh_node));
    std::memcpy(prim_index_out, bld.idx.data(), (size_t)n * sizeof(uint32_t));
    *num_nodes_out = (uint32_t)bld.nodes.size();
    if (depth_out) *depth_out = bld.depth;
    return TRACER_OK;
}

extern "C" int tracer_validate_bvh(int prim_type, const void* prims, uint32_t n, const tracer_bvh_node* nodes,
                                   uint32_t num_nodes, const uint32_t* prim_index, uint32_t* depth_out)
{
    if (!prims || !nodes || !prim_index || n == 0 || num_nodes == 0) return TRACER_ERR_BAD_BVH;
    if (prim_type != TRACER_PRIM_TRIANGLE && prim_type != TRACER_PRIM_SPHERE) return TRACER_ERR_INVALID_ARG;
    std::vector<Prim> p = make_prims(prim_type, prims, n);
    std::vector<uint32_t> seen(n, 0);
    std::vector<uint8_t> visited(num_nodes, 0);
    struct Item {
        uint32_t node, level;
    };
    std::vector<Item> todo{{0, 1}};
    uint32_t depth = 0;
    auto contains = [](const tracer_bvh_node& o, const Box& b) {
        for (int a = 0; a < 3; ++a)
            if (!((double)o.bmin[a] <= b.lo[a] && b.hi[a] <= (double)o.bmax[a])) return false;
        return true;
    };
    while (!todo.empty()) {
        Item it = todo.back();
        todo.pop_back();
        if (it.node >= num_nodes || visited[it.node]) return TRACER_ERR_BAD_BVH;
        visited[it.node] = 1;
        depth = std::max(depth, it.level);
        if (it.level > 1024) return TRACER_ERR_BAD_BVH;
        const tracer_bvh_node& nd = nodes[it.node];
        if (nd.count > 0) {
            int64_t f = nd.left_or_first, c = nd.count;
            if (f < 0 || f + c > (int64_t)n) return TRACER_ERR_BAD_BVH;
            for (int64_t k = f; k < f + c; ++k) {
                uint32_t pi = prim_index[k];
                if (pi >= n) return TRACER_ERR_BAD_BVH;
                seen[pi]++;
                if (!contains(nd, p[pi].box)) return TRACER_ERR_BAD_BVH;
            }
        } else if (nd.count == 0) {
            int64_t l = nd.left_or_first;
            if (l <= 0 || l + 1 >= (int64_t)num_nodes) return TRACER_ERR_BAD_BVH;
            for (int k = 0; k < 2; ++k) {
                const tracer_bvh_node& c = nodes[l + k];
                Box cb;
                for (int a = 0; a < 3; ++a) {
                    cb.lo[a] = c.bmin[a];
                    cb.hi[a] = c.bmax[a];
                }
                if (!contains(nd, cb)) return TRACER_ERR_BAD_BVH;
                todo.push_back({(uint32_t)(l + k), it.level + 1});
            }
        } else {
            return TRACER_ERR_BAD_BVH;
        }
    }
    for (uint32_t i = 0; i < n; ++i)
        if (seen[i] != 1) return TRACER_ERR_BAD_BVH;
    if (depth_out) *depth_out = depth;
    return TRACER_OK;
}
