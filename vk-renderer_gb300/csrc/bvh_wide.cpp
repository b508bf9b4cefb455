// Collapse of a binary BVH into 4-wide nodes (see bvh_wide.h).  Host code;
// deterministic (ties in surface area keep the first child in order).
#include "bvh_wide.h"

#include <cmath>
#include <limits>
#include <utility>

namespace vkt {

namespace {

double surface_area(const tracer_bvh_node& n)
{
    const double dx = (double)n.bmax[0] - n.bmin[0];
    const double dy = (double)n.bmax[1] - n.bmin[1];
    const double dz = (double)n.bmax[2] - n.bmin[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

bool leaf_code(const tracer_bvh_node& n, int32_t& code)
{
    if (n.count < 1 || n.count > 64 || n.left_or_first < 0 || n.left_or_first >= (1 << 25)) return false;
    code = -1 - ((n.left_or_first << 6) | (n.count - 1));
    return true;
}

void set_child(WideNode& w, int k, const tracer_bvh_node& n, int32_t ref)
{
    WideChild& c = w.c[k];
    for (int a = 0; a < 3; ++a) {
        c.lo[a] = n.bmin[a];
        c.hi[a] = n.bmax[a];
    }
    c.ref = ref;
    c.pad = 0;
}

WideNode empty_node()
{
    WideNode w;
    const float inf = std::numeric_limits<float>::infinity();
    for (int k = 0; k < 4; ++k) {
        for (int a = 0; a < 3; ++a) {
            w.c[k].lo[a] = inf;
            w.c[k].hi[a] = -inf;
        }
        w.c[k].ref = 0;
        w.c[k].pad = 0;
    }
    return w;
}

}  // namespace

bool encode_refs(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<tracer_bvh_node>& out)
{
    out.assign(nodes, nodes + num_nodes);
    for (uint32_t i = 0; i < num_nodes; ++i) {
        int32_t ref = nodes[i].left_or_first;
        if (nodes[i].count > 0 && !leaf_code(nodes[i], ref)) return false;
        out[i].left_or_first = ref;
        out[i].count = 0;
    }
    return true;
}

bool collapse_wide4(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<WideNode>& out,
                    uint32_t* depth_out)
{
    out.clear();
    if (depth_out) *depth_out = 0;
    if (!nodes || num_nodes == 0) return true;
    out.push_back(empty_node());
    // work list: (wide node index, binary node it expands, wide level)
    std::vector<std::pair<uint32_t, uint32_t>> work{{0u, 0u}};
    std::vector<uint32_t> level{1};
    uint32_t depth = 1;
    for (size_t wi = 0; wi < work.size(); ++wi) {
        const uint32_t w = work[wi].first, b = work[wi].second;
        const uint32_t lev = level[wi];
        std::vector<uint32_t> kids;
        if (nodes[b].count > 0) {
            kids.push_back(b);  // a leaf root: one leaf child
        } else {
            kids.push_back((uint32_t)nodes[b].left_or_first);
            kids.push_back((uint32_t)nodes[b].left_or_first + 1);
            while (kids.size() < 4) {
                int best = -1;
                double best_area = -1.0;
                for (size_t k = 0; k < kids.size(); ++k) {
                    const tracer_bvh_node& n = nodes[kids[k]];
                    if (n.count > 0) continue;
                    const double a = surface_area(n);
                    if (a > best_area) {
                        best_area = a;
                        best = (int)k;
                    }
                }
                if (best < 0) break;
                const uint32_t e = kids[best];
                kids[best] = (uint32_t)nodes[e].left_or_first;
                kids.insert(kids.begin() + best + 1, (uint32_t)nodes[e].left_or_first + 1);
            }
        }
        for (size_t k = 0; k < kids.size(); ++k) {
            const uint32_t c = kids[k];
            if (c >= num_nodes) return false;
            const tracer_bvh_node& n = nodes[c];
            int32_t ref;
            if (n.count > 0) {
                if (!leaf_code(n, ref)) return false;
            } else {
                ref = (int32_t)out.size();
                out.push_back(empty_node());
                work.push_back({(uint32_t)ref, c});
                level.push_back(lev + 1);
                if (lev + 1 > depth) depth = lev + 1;
            }
            set_child(out[w], (int)k, n, ref);
        }
    }
    if (depth_out) *depth_out = depth;
    return true;
}

}  // namespace vkt
