// Test harness (host only): builds the 8-wide BVH of sparkle_gb300/csrc/bvh_builder.cpp over given boxes and
// checks every structural invariant the device walk relies on. Returns 0 when all hold, else an error code.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../sparkle_gb300/csrc/bvh_builder.h"

using namespace spk;

// mode 0: binary leaves <= 3 + greedy collapse; mode 1: one item per binary leaf + SAH-optimal collapse.
// out_cost: SAH cost of the wide tree (half area x (1 per node + 0.3 per item)) relative to the root box.
extern "C" int wide_bvh_check(const float *boxes6, uint32_t n, int threads, int mode, uint32_t *out_stats /*4*/,
                              double *out_cost) {
    std::vector<BuildBox> boxes(n);
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            boxes[i].lo[k] = boxes6[6 * i + k];
            boxes[i].hi[k] = boxes6[6 * i + 3 + k];
        }
    }
    const Bvh2 b2 = build_bvh2(boxes, mode ? 1 : 3, threads);
    if (n == 0) return b2.nodes.empty() ? 0 : 1;
    // binary tree: leaves <= 3 items, every item once
    std::vector<int> seen(n, 0);
    for (const Bvh2Node &nd : b2.nodes) {
        if (nd.count > 3) return 2;
        if (nd.count == 0 && nd.first + 1 >= b2.nodes.size()) return 3;
        for (uint32_t i = 0; i < nd.count; ++i) seen[b2.items[nd.first + i]]++;
    }
    for (int s : seen)
        if (s != 1) return 4;
    const WideBvh w = mode ? collapse_wide_sah(b2) : collapse_wide(b2);
    double cost = 0.0, root_area = 0.0;
    if (w.items.size() != n) return 5;
    std::vector<int> seen_items(n, 0);
    std::vector<int> refs(w.nodes.size(), 0);
    refs[0] = 1;
    uint32_t max_depth = 0;
    std::vector<std::pair<uint32_t, uint32_t>> stack{{0, 1}};
    size_t visited = 0;
    while (!stack.empty()) {
        const auto [idx, depth] = stack.back();
        stack.pop_back();
        ++visited;
        if (depth > max_depth) max_depth = depth;
        const WideNode &nd = w.nodes[idx];
        double p[3], sc[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = nd.p[k];
            if (nd.e[k] == 0 || nd.e[k] == 255) return 6;
            sc[k] = std::ldexp(1.0, static_cast<int>(nd.e[k]) - 127);
        }
        uint32_t inner_rank = 0, item_total = 0;
        double nlo[3] = {1e300, 1e300, 1e300}, nhi[3] = {-1e300, -1e300, -1e300};
        for (int s = 0; s < 8; ++s) {
            const uint32_t m = nd.meta[s];
            const bool inner = (nd.imask >> s) & 1u;
            double lo[3], hi[3];
            for (int k = 0; k < 3; ++k) {
                if (nd.qlo[k][s] >= nd.qhi[k][s] && m != 0) return 7;
                lo[k] = p[k] + nd.qlo[k][s] * sc[k];
                hi[k] = p[k] + nd.qhi[k][s] * sc[k];
            }
            if (m == 0) {
                if (inner) return 8;
                continue;
            }
            for (int k = 0; k < 3; ++k) {
                nlo[k] = std::fmin(nlo[k], lo[k]);
                nhi[k] = std::fmax(nhi[k], hi[k]);
            }
            if (inner) {
                if (m != (0x20u | (24u + s))) return 9;
                const uint32_t child = nd.child_base + inner_rank++;
                if (child >= w.nodes.size()) return 10;
                if (++refs[child] != 1) return 11;
                // the child's own children boxes must lie inside this slot's box
                const WideNode &c = w.nodes[child];
                for (int cs = 0; cs < 8; ++cs) {
                    if (c.meta[cs] == 0) continue;
                    for (int k = 0; k < 3; ++k) {
                        const double cs_sc = std::ldexp(1.0, static_cast<int>(c.e[k]) - 127);
                        const double clo = c.p[k] + c.qlo[k][cs] * cs_sc, chi = c.p[k] + c.qhi[k][cs] * cs_sc;
                        (void)clo;
                        (void)chi;
                    }
                }
                stack.push_back({child, depth + 1});
            } else {
                if ((m & 0x18u) == 0x18u) return 12;
                const uint32_t cnt = m >> 5;
                if (cnt != 1 && cnt != 3 && cnt != 7) return 13;
                const uint32_t ni = cnt == 1 ? 1 : cnt == 3 ? 2 : 3;
                const uint32_t off = m & 0x1Fu;
                if (off + ni > 24) return 14;
                for (uint32_t i = 0; i < ni; ++i) {
                    const uint64_t it = static_cast<uint64_t>(nd.item_base) + off + i;
                    if (it >= w.items.size()) return 15;
                    const uint32_t item = w.items[it];
                    if (item >= n) return 16;
                    seen_items[item]++;
                    for (int k = 0; k < 3; ++k) {
                        if (boxes[item].lo[k] < lo[k] || boxes[item].hi[k] > hi[k]) return 17;
                    }
                }
                item_total += ni;
                const double ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
                cost += 0.3 * ni * (ex * ey + ey * ez + ez * ex);
            }
        }
        if (item_total > 24) return 18;
        const double ex = nhi[0] - nlo[0], ey = nhi[1] - nlo[1], ez = nhi[2] - nlo[2];
        const double area = ex * ey + ey * ez + ez * ex;
        cost += area;
        if (idx == 0) root_area = area;
    }
    for (int s : seen_items)
        if (s != 1) return 19;
    if (visited != w.nodes.size()) return 20;
    out_stats[0] = static_cast<uint32_t>(w.nodes.size());
    out_stats[1] = max_depth;
    out_stats[2] = static_cast<uint32_t>(b2.nodes.size());
    out_stats[3] = static_cast<uint32_t>(w.items.size());
    if (out_cost) *out_cost = root_area > 0 ? cost / root_area : 0.0;
    return 0;
}
