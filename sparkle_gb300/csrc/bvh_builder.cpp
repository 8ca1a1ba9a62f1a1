// bvh_builder.cpp -- binned-SAH BVH2 and its collapse into 8-wide quantised nodes (see bvh_builder.h).
#include "bvh_builder.h"

#include <algorithm>
#include <functional>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <limits>
#include <mutex>
#include <thread>

namespace spk {
namespace {

#ifndef SPK_SAH_BINS
#define SPK_SAH_BINS 32  // SAH bins per axis of the binned host build
#endif
constexpr int kBins = SPK_SAH_BINS;

inline void box_reset(BuildBox &b) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::numeric_limits<float>::max();
        b.hi[k] = -std::numeric_limits<float>::max();
    }
}
inline void box_grow(BuildBox &b, const BuildBox &o) {
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], o.lo[k]);
        b.hi[k] = std::max(b.hi[k], o.hi[k]);
    }
}
inline float box_half_area(const BuildBox &b) {
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = std::max(0.f, b.hi[k] - b.lo[k]);
    return d[0] * d[1] + d[1] * d[2] + d[2] * d[0];
}

struct Builder {
    const std::vector<BuildBox> &boxes;
    std::vector<float> cx, cy, cz;
    std::vector<uint32_t> &items;
    uint32_t max_leaf;

    // Subtrees are built into private node vectors and spliced, so independent halves run on threads.
    struct Sub {
        std::vector<Bvh2Node> nodes;
    };

    const float *centroid(int axis) const { return axis == 0 ? cx.data() : axis == 1 ? cy.data() : cz.data(); }

    // Builds the subtree over items[begin, end) into sub.nodes (root at index `root`).
    void build(Sub &sub, uint32_t root, uint32_t begin, uint32_t end, int depth, int spawn_depth) {
        struct Task {
            uint32_t node, begin, end;
            int depth;
        };
        std::vector<Task> work{{root, begin, end, depth}};
        std::vector<std::future<std::pair<uint32_t, Sub>>> pending;
        while (!work.empty()) {
            const Task t = work.back();
            work.pop_back();
            BuildBox nb, cb;
            box_reset(nb);
            box_reset(cb);
            for (uint32_t i = t.begin; i < t.end; ++i) {
                const uint32_t p = items[i];
                box_grow(nb, boxes[p]);
                const BuildBox c{{cx[p], cy[p], cz[p]}, {cx[p], cy[p], cz[p]}};
                box_grow(cb, c);
            }
            Bvh2Node node{};
            for (int k = 0; k < 3; ++k) {
                node.lo[k] = nb.lo[k];
                node.hi[k] = nb.hi[k];
            }
            const uint32_t count = t.end - t.begin;
            float best_cost = std::numeric_limits<float>::max();
            int best_axis = -1, best_split = -1;
            if (count > 1) {
                for (int axis = 0; axis < 3; ++axis) {
                    const float lo = cb.lo[axis], ext = cb.hi[axis] - cb.lo[axis];
                    if (!(ext > 0.f)) continue;
                    const float scale = kBins / ext;
                    BuildBox bb[kBins];
                    uint32_t bc[kBins] = {};
                    for (auto &b : bb) box_reset(b);
                    const float *c = centroid(axis);
                    for (uint32_t i = t.begin; i < t.end; ++i) {
                        const uint32_t p = items[i];
                        const int bi = std::min(kBins - 1, std::max(0, static_cast<int>((c[p] - lo) * scale)));
                        bc[bi]++;
                        box_grow(bb[bi], boxes[p]);
                    }
                    float ra[kBins];
                    uint32_t rc[kBins];
                    BuildBox acc;
                    box_reset(acc);
                    uint32_t cnt = 0;
                    for (int b = kBins - 1; b > 0; --b) {
                        box_grow(acc, bb[b]);
                        cnt += bc[b];
                        ra[b] = box_half_area(acc);
                        rc[b] = cnt;
                    }
                    box_reset(acc);
                    cnt = 0;
                    for (int b = 0; b < kBins - 1; ++b) {
                        box_grow(acc, bb[b]);
                        cnt += bc[b];
                        if (cnt == 0 || rc[b + 1] == 0) continue;
                        const float cost = box_half_area(acc) * cnt + ra[b + 1] * rc[b + 1];
                        if (cost < best_cost) {
                            best_cost = cost;
                            best_axis = axis;
                            best_split = b;
                        }
                    }
                }
            }
            const float leaf_cost = box_half_area(nb) * count;
            const float split_cost = box_half_area(nb) + best_cost;
            if (count == 1 || (count <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost))) {
                node.first = t.begin;
                node.count = count;
                sub.nodes[t.node] = node;
                continue;
            }
            uint32_t mid;
            if (best_axis < 0) {
                mid = t.begin + count / 2;
            } else {
                const float lo = cb.lo[best_axis], scale = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
                const float *c = centroid(best_axis);
                auto it = std::partition(items.begin() + t.begin, items.begin() + t.end, [&](uint32_t p) {
                    const int bi = std::min(kBins - 1, std::max(0, static_cast<int>((c[p] - lo) * scale)));
                    return bi <= best_split;
                });
                mid = static_cast<uint32_t>(it - items.begin());
                if (mid == t.begin || mid == t.end) mid = t.begin + count / 2;
            }
            const uint32_t left = static_cast<uint32_t>(sub.nodes.size());
            node.first = left;
            node.count = 0;
            sub.nodes[t.node] = node;
            sub.nodes.push_back({});
            sub.nodes.push_back({});
            const uint32_t big = 1u << 16;
            if (t.depth < spawn_depth && (mid - t.begin) >= big && (t.end - mid) >= big) {
                // Right half on another thread into its own node vector; spliced after the join.
                const uint32_t rb = mid, re = t.end;
                const int d = t.depth + 1;
                pending.push_back(std::async(std::launch::async, [this, rb, re, d, spawn_depth, left]() {
                    Sub s;
                    s.nodes.reserve(2 * (re - rb));
                    s.nodes.push_back({});
                    build(s, 0, rb, re, d, spawn_depth);
                    return std::make_pair(left + 1, std::move(s));
                }));
            } else {
                work.push_back({left + 1, mid, t.end, t.depth + 1});
            }
            work.push_back({left, t.begin, mid, t.depth + 1});
        }
        for (auto &f : pending) {
            auto res = f.get();
            const uint32_t slot = res.first;
            Sub &s = res.second;
            const uint32_t offset = static_cast<uint32_t>(sub.nodes.size()) - 1;  // s.nodes[0] goes to `slot`
            auto fix = [&](Bvh2Node n) {
                if (n.count == 0) n.first += offset;
                return n;
            };
            sub.nodes[slot] = fix(s.nodes[0]);
            for (size_t k = 1; k < s.nodes.size(); ++k) sub.nodes.push_back(fix(s.nodes[k]));
        }
    }
};

// ----------------------------------------------------------------------------------------------
// Collapse
// ----------------------------------------------------------------------------------------------

inline float node_half_area(const Bvh2Node &n) {
    const BuildBox b{{n.lo[0], n.lo[1], n.lo[2]}, {n.hi[0], n.hi[1], n.hi[2]}};
    return box_half_area(b);
}

void quantize_node(WideNode &w, const Bvh2Node *const *child, int nchild, const int *slot_of) {
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = std::numeric_limits<double>::max();
        hi[k] = -std::numeric_limits<double>::max();
    }
    for (int c = 0; c < nchild; ++c) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], static_cast<double>(child[c]->lo[k]));
            hi[k] = std::max(hi[k], static_cast<double>(child[c]->hi[k]));
        }
    }
    for (int k = 0; k < 3; ++k) {
        w.p[k] = static_cast<float>(lo[k]);
        if (static_cast<double>(w.p[k]) > lo[k]) w.p[k] = std::nextafter(w.p[k], -std::numeric_limits<float>::max());
        const double origin = w.p[k];
        const double ext = hi[k] - origin;
        int e = ext > 0 ? static_cast<int>(std::ceil(std::log2(ext / 255.0))) : -126;
        e = std::max(-126, std::min(127, e));
        while (e < 127 && std::ldexp(255.0, e) < ext) ++e;
        w.e[k] = static_cast<uint8_t>(e + 127);
        const double scale = std::ldexp(1.0, e);
        for (int c = 0; c < nchild; ++c) {
            const int s = slot_of[c];
            double ql = std::floor((static_cast<double>(child[c]->lo[k]) - origin) / scale);
            double qh = std::ceil((static_cast<double>(child[c]->hi[k]) - origin) / scale);
            ql = std::max(0.0, std::min(255.0, ql));
            qh = std::max(0.0, std::min(255.0, qh));
            if (qh <= ql) {  // give every child a non-zero extent so a flat box is never missed by rounding
                if (qh < 255.0) {
                    qh = ql + 1.0;
                } else {
                    ql = qh - 1.0;
                }
            }
            w.qlo[k][s] = static_cast<uint8_t>(ql);
            w.qhi[k][s] = static_cast<uint8_t>(qh);
        }
    }
}

}  // namespace

Bvh2 build_bvh2(const std::vector<BuildBox> &boxes, uint32_t max_leaf, int num_threads) {
    Bvh2 out;
    const uint32_t n = static_cast<uint32_t>(boxes.size());
    if (n == 0) return out;
    out.items.resize(n);
    for (uint32_t i = 0; i < n; ++i) out.items[i] = i;
    Builder b{boxes, {}, {}, {}, out.items, std::max(1u, std::min(max_leaf, 3u))};
    b.cx.resize(n);
    b.cy.resize(n);
    b.cz.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        b.cx[i] = 0.5f * (boxes[i].lo[0] + boxes[i].hi[0]);
        b.cy[i] = 0.5f * (boxes[i].lo[1] + boxes[i].hi[1]);
        b.cz[i] = 0.5f * (boxes[i].lo[2] + boxes[i].hi[2]);
    }
    int spawn_depth = 0;
    for (int t = 1; t < num_threads; t *= 2) ++spawn_depth;
    Builder::Sub root;
    root.nodes.reserve(2 * static_cast<size_t>(n));
    root.nodes.push_back({});
    b.build(root, 0, 0, n, 0, spawn_depth);
    out.nodes = std::move(root.nodes);
    return out;
}

WideBvh collapse_wide(const Bvh2 &bvh, int max_children) {
    max_children = std::max(2, std::min(8, max_children));
    WideBvh out;
    if (bvh.nodes.empty()) return out;
    out.nodes.reserve(bvh.nodes.size() / 4 + 1);
    out.items.reserve(bvh.items.size());
    out.nodes.push_back(WideNode{});
    struct Job {
        uint32_t bvh_node, wide_node;
    };
    std::vector<Job> queue{{0, 0}};
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const Job job = queue[qi];
        const Bvh2Node &root = bvh.nodes[job.bvh_node];
        // Open the binary subtree until max_children children: always expand the inner child of largest area.
        std::vector<uint32_t> kids;
        if (root.count > 0) {
            kids.push_back(job.bvh_node);  // a leaf root becomes a node with a single leaf child
        } else {
            kids.push_back(root.first);
            kids.push_back(root.first + 1);
            while (static_cast<int>(kids.size()) < max_children) {
                int best = -1;
                float best_area = -1.f;
                for (size_t k = 0; k < kids.size(); ++k) {
                    const Bvh2Node &c = bvh.nodes[kids[k]];
                    if (c.count == 0 && node_half_area(c) > best_area) {
                        best_area = node_half_area(c);
                        best = static_cast<int>(k);
                    }
                }
                if (best < 0) break;
                const uint32_t f = bvh.nodes[kids[best]].first;
                kids[best] = f;
                kids.push_back(f + 1);
            }
        }
        const int nk = static_cast<int>(kids.size());
        // Octant slot assignment: slot s is the near-most child for rays whose sign bits equal s.
        float pc[3];
        {
            float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                           std::numeric_limits<float>::max()};
            float hi[3] = {-lo[0], -lo[1], -lo[2]};
            for (uint32_t k : kids) {
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], bvh.nodes[k].lo[a]);
                    hi[a] = std::max(hi[a], bvh.nodes[k].hi[a]);
                }
            }
            for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (lo[a] + hi[a]);
        }
        struct Cost {
            float c;
            int kid, slot;
        };
        std::vector<Cost> costs;
        for (int k = 0; k < nk; ++k) {
            const Bvh2Node &c = bvh.nodes[kids[k]];
            float d[3];
            for (int a = 0; a < 3; ++a) d[a] = 0.5f * (c.lo[a] + c.hi[a]) - pc[a];
            for (int s = 0; s < 8; ++s) {
                const float v = (s & 1 ? -d[0] : d[0]) + (s & 2 ? -d[1] : d[1]) + (s & 4 ? -d[2] : d[2]);
                costs.push_back({v, k, s});
            }
        }
        std::stable_sort(costs.begin(), costs.end(), [](const Cost &a, const Cost &b) { return a.c < b.c; });
        int slot_of[8], kid_in_slot[8];
        std::fill(slot_of, slot_of + 8, -1);
        std::fill(kid_in_slot, kid_in_slot + 8, -1);
        for (const Cost &c : costs) {
            if (slot_of[c.kid] < 0 && kid_in_slot[c.slot] < 0) {
                slot_of[c.kid] = c.slot;
                kid_in_slot[c.slot] = c.kid;
            }
        }
        WideNode w{};
        const Bvh2Node *child_ptrs[8];
        for (int k = 0; k < nk; ++k) child_ptrs[k] = &bvh.nodes[kids[k]];
        quantize_node(w, child_ptrs, nk, slot_of);
        // Inner children get consecutive node indices in slot order; leaf items go to consecutive item slots.
        w.child_base = static_cast<uint32_t>(out.nodes.size());
        w.item_base = static_cast<uint32_t>(out.items.size());
        uint32_t offset = 0;
        for (int s = 0; s < 8; ++s) {
            const int k = kid_in_slot[s];
            if (k < 0) {
                w.meta[s] = 0;
                continue;
            }
            const Bvh2Node &c = bvh.nodes[kids[k]];
            if (c.count == 0) {
                w.imask |= static_cast<uint8_t>(1u << s);
                w.meta[s] = static_cast<uint8_t>(0x20u | (24u + s));
                queue.push_back({kids[k], static_cast<uint32_t>(out.nodes.size())});
                out.nodes.push_back(WideNode{});
            } else {
                const uint32_t unary = (1u << c.count) - 1u;
                w.meta[s] = static_cast<uint8_t>((unary << 5) | offset);
                for (uint32_t i = 0; i < c.count; ++i) out.items.push_back(bvh.items[c.first + i]);
                offset += c.count;
            }
        }
        out.nodes[job.wide_node] = w;
    }
    return out;
}


namespace {

#ifndef SPK_SAH_ITEM_COST
#define SPK_SAH_ITEM_COST 0.3f  // cost of testing one leaf item relative to one wide-node visit
#endif
constexpr float kSahNodeCost = 1.0f;
constexpr float kSahItemCost = SPK_SAH_ITEM_COST;

// Assigns the children of one wide node to octant slots (slot s = near-most child for rays whose sign
// bits equal s) and writes its quantised boxes: the same assignment collapse_wide uses.
void assign_slots(const Bvh2 &bvh, const std::vector<uint32_t> &kids, int *slot_of, int *kid_in_slot) {
    const int nk = static_cast<int>(kids.size());
    float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                   std::numeric_limits<float>::max()};
    float hi[3] = {-lo[0], -lo[1], -lo[2]};
    for (uint32_t k : kids)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], bvh.nodes[k].lo[a]);
            hi[a] = std::max(hi[a], bvh.nodes[k].hi[a]);
        }
    float pc[3];
    for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (lo[a] + hi[a]);
    struct Cost {
        float c;
        int kid, slot;
    };
    std::vector<Cost> costs;
    for (int k = 0; k < nk; ++k) {
        const Bvh2Node &c = bvh.nodes[kids[k]];
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = 0.5f * (c.lo[a] + c.hi[a]) - pc[a];
        for (int sl = 0; sl < 8; ++sl) {
            const float v = (sl & 1 ? -d[0] : d[0]) + (sl & 2 ? -d[1] : d[1]) + (sl & 4 ? -d[2] : d[2]);
            costs.push_back({v, k, sl});
        }
    }
    std::stable_sort(costs.begin(), costs.end(), [](const Cost &a, const Cost &b) { return a.c < b.c; });
    std::fill(slot_of, slot_of + 8, -1);
    std::fill(kid_in_slot, kid_in_slot + 8, -1);
    for (const Cost &c : costs) {
        if (slot_of[c.kid] < 0 && kid_in_slot[c.slot] < 0) {
            slot_of[c.kid] = c.slot;
            kid_in_slot[c.slot] = c.kid;
        }
    }
}

}  // namespace

WideBvh collapse_wide_sah(const Bvh2 &bvh, int max_children, int max_leaf) {
    const int K = std::max(2, std::min(8, max_children));
    max_leaf = std::max(1, std::min(3, max_leaf));
    WideBvh out;
    const size_t n = bvh.nodes.size();
    if (n == 0) return out;
    // Post-order of the binary tree (explicit stack: trees over millions of items are deep).
    std::vector<uint32_t> order;
    order.reserve(n);
    {
        std::vector<std::pair<uint32_t, bool>> st{{0u, false}};
        while (!st.empty()) {
            auto [v, expanded] = st.back();
            st.pop_back();
            const Bvh2Node &b = bvh.nodes[v];
            if (b.count > 0 || expanded) {
                order.push_back(v);
                continue;
            }
            st.push_back({v, true});
            st.push_back({b.first + 1, false});
            st.push_back({b.first, false});
        }
    }
    const float kInf = std::numeric_limits<float>::infinity();
    std::vector<uint32_t> items_in(n, 0);
    std::vector<float> cost(n * 9, kInf);     // cost[v * 9 + i], i = 1..K: best with at most i roots
    std::vector<uint8_t> split(n * 9, 0);     // split[v * 9 + j]: left share k of the best j-root distribution
    std::vector<uint8_t> use_dist(n * 9, 0);  // use_dist[v * 9 + i]: at most i roots uses the distribution
    std::vector<uint8_t> leaf_root(n, 0);     // the single-root option is a leaf
    for (uint32_t v : order) {
        const Bvh2Node &b = bvh.nodes[v];
        const float area = node_half_area(b);
        float *C = &cost[static_cast<size_t>(v) * 9];
        if (b.count > 0) {
            items_in[v] = b.count;
            const float leaf = b.count <= static_cast<uint32_t>(max_leaf) ? area * kSahItemCost * b.count : kInf;
            for (int i = 1; i <= K; ++i) C[i] = leaf;
            leaf_root[v] = 1;
            continue;
        }
        const uint32_t L = b.first, R = b.first + 1;
        items_in[v] = items_in[L] + items_in[R];
        const float *CL = &cost[static_cast<size_t>(L) * 9];
        const float *CR = &cost[static_cast<size_t>(R) * 9];
        float dist[9];
        for (int j = 2; j <= K; ++j) {
            float best = kInf;
            int bk = 1;
            for (int k = 1; k < j; ++k) {
                const float c = CL[k] + CR[j - k];
                if (c < best) {
                    best = c;
                    bk = k;
                }
            }
            dist[j] = best;
            split[static_cast<size_t>(v) * 9 + j] = static_cast<uint8_t>(bk);
        }
        const float leaf =
            items_in[v] <= static_cast<uint32_t>(max_leaf) ? area * kSahItemCost * items_in[v] : kInf;
        const float inner = area * kSahNodeCost + dist[K];
        leaf_root[v] = leaf <= inner ? 1 : 0;
        C[1] = std::min(leaf, inner);
        for (int i = 2; i <= K; ++i) {
            if (dist[i] < C[i - 1]) {
                C[i] = dist[i];
                use_dist[static_cast<size_t>(v) * 9 + i] = 1;
            } else {
                C[i] = C[i - 1];
            }
        }
    }
    // Roots of the best representation of subtree v with at most i roots.
    std::function<void(uint32_t, int, std::vector<uint32_t> &)> roots = [&](uint32_t v, int i,
                                                                          std::vector<uint32_t> &outv) {
        while (i > 1 && !use_dist[static_cast<size_t>(v) * 9 + i]) --i;
        if (i == 1) {
            outv.push_back(v);
            return;
        }
        const int k = split[static_cast<size_t>(v) * 9 + i];
        roots(bvh.nodes[v].first, k, outv);
        roots(bvh.nodes[v].first + 1, i - k, outv);
    };
    auto collect_items = [&](uint32_t v, std::vector<uint32_t> &dst) {
        std::vector<uint32_t> st{v};
        while (!st.empty()) {
            const uint32_t u = st.back();
            st.pop_back();
            const Bvh2Node &b = bvh.nodes[u];
            if (b.count > 0) {
                for (uint32_t t = 0; t < b.count; ++t) dst.push_back(bvh.items[b.first + t]);
            } else {
                st.push_back(b.first + 1);
                st.push_back(b.first);
            }
        }
    };
    out.nodes.reserve(n / 4 + 1);
    out.items.reserve(bvh.items.size());
    out.nodes.push_back(WideNode{});
    struct Job {
        uint32_t bvh_node, wide_node;
    };
    std::vector<Job> queue{{0, 0}};
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const Job job = queue[qi];
        std::vector<uint32_t> kids;
        if (leaf_root[job.bvh_node]) {
            kids.push_back(job.bvh_node);  // the whole tree is one leaf: a node with a single leaf child
        } else {
            const Bvh2Node &b = bvh.nodes[job.bvh_node];
            const int k = split[static_cast<size_t>(job.bvh_node) * 9 + K];
            roots(b.first, k, kids);
            roots(b.first + 1, K - k, kids);
        }
        int slot_of[8], kid_in_slot[8];
        assign_slots(bvh, kids, slot_of, kid_in_slot);
        WideNode w{};
        const Bvh2Node *child_ptrs[8];
        for (size_t k = 0; k < kids.size(); ++k) child_ptrs[k] = &bvh.nodes[kids[k]];
        quantize_node(w, child_ptrs, static_cast<int>(kids.size()), slot_of);
        w.child_base = static_cast<uint32_t>(out.nodes.size());
        w.item_base = static_cast<uint32_t>(out.items.size());
        uint32_t offset = 0;
        for (int sl = 0; sl < 8; ++sl) {
            const int k = kid_in_slot[sl];
            if (k < 0) {
                w.meta[sl] = 0;
                continue;
            }
            const uint32_t c = kids[k];
            const bool as_leaf = leaf_root[c] || (kids.size() == 1 && kids[0] == job.bvh_node);
            if (!as_leaf) {
                w.imask |= static_cast<uint8_t>(1u << sl);
                w.meta[sl] = static_cast<uint8_t>(0x20u | (24u + sl));
                queue.push_back({c, static_cast<uint32_t>(out.nodes.size())});
                out.nodes.push_back(WideNode{});
            } else {
                std::vector<uint32_t> its;
                collect_items(c, its);
                const uint32_t cnt = static_cast<uint32_t>(its.size());
                const uint32_t unary = (1u << cnt) - 1u;
                w.meta[sl] = static_cast<uint8_t>((unary << 5) | offset);
                for (uint32_t it : its) out.items.push_back(it);
                offset += cnt;
            }
        }
        out.nodes[job.wide_node] = w;
    }
    return out;
}

}  // namespace spk
