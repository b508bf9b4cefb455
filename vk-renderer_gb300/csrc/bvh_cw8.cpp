// Collapse of a binary BVH into compressed 8-wide nodes (see bvh_cw8.h).
// Host code, deterministic: every choice has a total order (surface area,
// then position in the child list; assignment scores, then child, then slot).
#include "bvh_cw8.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace vkt {

namespace {

double area(const tracer_bvh_node& n)
{
    const double dx = (double)n.bmax[0] - n.bmin[0];
    const double dy = (double)n.bmax[1] - n.bmin[1];
    const double dz = (double)n.bmax[2] - n.bmin[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}

bool is_leaf(const tracer_bvh_node& n) { return n.count > 0; }

// Smallest e (biased float exponent, 1..254) with 2^(e - 127) * 255 >= ext.
int grid_exponent(double ext)
{
    int e = 1;  // 2^-126
    while (e < 254 && std::ldexp(255.0, e - 127) < ext) ++e;
    return e;
}

void put_byte(uint32_t* w, int k, uint32_t v)
{
    w[k / 4] |= (v & 0xFFu) << (8 * (k % 4));
}

}  // namespace

bool build_cw8(const tracer_bvh_node* nodes, uint32_t num_nodes, std::vector<Cw8Node>& out,
               std::vector<uint32_t>& order_out, uint32_t* depth_out)
{
    out.clear();
    order_out.clear();
    if (depth_out) *depth_out = 0;
    if (!nodes || num_nodes == 0) return true;
    for (uint32_t i = 0; i < num_nodes; ++i) {
        const tracer_bvh_node& n = nodes[i];
        if (n.count < 0 || (uint32_t)n.count > kCw8MaxLeafPrims) return false;
        if (n.count == 0 && (n.left_or_first <= 0 || (uint32_t)n.left_or_first + 1 >= num_nodes)) return false;
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs(n.bmin[a]) <= 1e6f && std::fabs(n.bmax[a]) <= 1e6f)) return false;
    }
    struct Work {
        uint32_t wide, bin, level;
    };
    std::vector<Work> work{{0u, 0u, 1u}};
    out.push_back(Cw8Node{});
    uint32_t depth = 1;
    for (size_t wi = 0; wi < work.size(); ++wi) {
        const Work W = work[wi];
        depth = std::max(depth, W.level);
        // children: the binary node's two (or the root leaf itself), expanded
        std::vector<uint32_t> kids;
        uint32_t prims = 0;
        if (is_leaf(nodes[W.bin])) {
            kids.push_back(W.bin);
            prims = (uint32_t)nodes[W.bin].count;
        } else {
            for (uint32_t c = 0; c < 2; ++c) {
                const uint32_t k = (uint32_t)nodes[W.bin].left_or_first + c;
                kids.push_back(k);
                if (is_leaf(nodes[k])) prims += (uint32_t)nodes[k].count;
            }
            while (kids.size() < 8) {
                int best = -1;
                double best_area = -1.0;
                uint32_t best_prims = 0;
                for (size_t k = 0; k < kids.size(); ++k) {
                    const tracer_bvh_node& n = nodes[kids[k]];
                    if (is_leaf(n)) continue;
                    uint32_t add = 0;
                    for (uint32_t c = 0; c < 2; ++c) {
                        const tracer_bvh_node& g = nodes[(uint32_t)n.left_or_first + c];
                        if (is_leaf(g)) add += (uint32_t)g.count;
                    }
                    if (prims + add > kCw8MaxNodePrims) continue;
                    const double a = area(n);
                    if (a > best_area) {
                        best_area = a;
                        best = (int)k;
                        best_prims = add;
                    }
                }
                if (best < 0) break;
                const uint32_t e = kids[best];
                kids[best] = (uint32_t)nodes[e].left_or_first;
                kids.insert(kids.begin() + best + 1, (uint32_t)nodes[e].left_or_first + 1);
                prims += best_prims;
            }
        }
        // slot assignment: slot s takes the child whose centroid lies furthest
        // toward the side where rays of octant s enter (greedy on the scores)
        double ulo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, uhi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        for (uint32_t k : kids)
            for (int a = 0; a < 3; ++a) {
                ulo[a] = std::min(ulo[a], (double)nodes[k].bmin[a]);
                uhi[a] = std::max(uhi[a], (double)nodes[k].bmax[a]);
            }
        const size_t nk = kids.size();
        std::vector<double> score(nk * 8);
        for (size_t k = 0; k < nk; ++k)
            for (int s = 0; s < 8; ++s) {
                double v = 0.0;
                for (int a = 0; a < 3; ++a) {
                    const double c = 0.5 * ((double)nodes[kids[k]].bmin[a] + nodes[kids[k]].bmax[a]) -
                                     0.5 * (ulo[a] + uhi[a]);
                    v += ((s >> a) & 1) ? c : -c;
                }
                score[k * 8 + s] = v;
            }
        int slot_of[8] = {-1, -1, -1, -1, -1, -1, -1, -1};  // child -> slot
        int kid_in[8] = {-1, -1, -1, -1, -1, -1, -1, -1};   // slot -> child
        for (size_t n = 0; n < nk; ++n) {
            int bk = -1, bs = -1;
            double bv = -HUGE_VAL;
            for (size_t k = 0; k < nk; ++k) {
                if (slot_of[k] >= 0) continue;
                for (int s = 0; s < 8; ++s) {
                    if (kid_in[s] >= 0) continue;
                    if (score[k * 8 + s] > bv) {
                        bv = score[k * 8 + s];
                        bk = (int)k;
                        bs = s;
                    }
                }
            }
            slot_of[bk] = bs;
            kid_in[bs] = bk;
        }
        // quantisation grid: origin = the union's low corner rounded down to
        // float, step = a power of two with 255 steps covering the union
        Cw8Node node{};
        float p[3];
        int ex[3];
        for (int a = 0; a < 3; ++a) {
            float f = (float)ulo[a];
            if ((double)f > ulo[a]) f = std::nextafter(f, -HUGE_VALF);
            p[a] = f;
            ex[a] = grid_exponent(uhi[a] - (double)f);
            std::memcpy(&node.w[a], &p[a], 4);
        }
        uint32_t imask = 0, n_int = 0;
        for (int s = 0; s < 8; ++s)
            if (kid_in[s] >= 0 && !is_leaf(nodes[kids[kid_in[s]]])) {
                imask |= 1u << s;
                ++n_int;
            }
        node.w[3] = (uint32_t)ex[0] | (uint32_t)ex[1] << 8 | (uint32_t)ex[2] << 16 | imask << 24;
        const uint32_t child_base = (uint32_t)out.size();
        const uint32_t prim_base = (uint32_t)order_out.size();
        node.w[4] = child_base;
        node.w[5] = prim_base;
        uint32_t next_child = child_base;
        for (int s = 0; s < 8; ++s) {
            if (kid_in[s] < 0) continue;
            const tracer_bvh_node& n = nodes[kids[kid_in[s]]];
            for (int a = 0; a < 3; ++a) {
                const double step = std::ldexp(1.0, ex[a] - 127);
                double qlo = std::floor(((double)n.bmin[a] - p[a]) / step);
                double qhi = std::ceil(((double)n.bmax[a] - p[a]) / step);
                qlo = std::min(255.0, std::max(0.0, qlo));
                qhi = std::min(255.0, std::max(0.0, qhi));
                // the decoded box must contain the child's box (exact in double)
                if (!((double)p[a] + qlo * step <= (double)n.bmin[a] && (double)p[a] + qhi * step >= (double)n.bmax[a]))
                    return false;
                put_byte(node.w + 8 + 2 * a, s, (uint32_t)qlo);
                put_byte(node.w + 14 + 2 * a, s, (uint32_t)qhi);
            }
            if (is_leaf(n)) {
                const uint32_t o = (uint32_t)order_out.size() - prim_base;
                put_byte(node.w + 20, s, (1u << n.count) - 1u);
                put_byte(node.w + 22, s, o);
                for (int32_t j = 0; j < n.count; ++j) order_out.push_back((uint32_t)(n.left_or_first + j));
            } else {
                put_byte(node.w + 6, s, 7u);
                put_byte(node.w + 20, s, 1u);
                put_byte(node.w + 22, s, 24u + (uint32_t)s);
                work.push_back({next_child++, kids[kid_in[s]], W.level + 1});
            }
        }
        if ((uint32_t)order_out.size() - prim_base > kCw8MaxNodePrims) return false;
        out[W.wide] = node;
        out.resize(out.size() + n_int);
    }
    if (depth_out) *depth_out = depth;
    return true;
}

}  // namespace vkt
