// batch_plan.h -- host-side plan of spk_render_batch (plain C++, no CUDA): the groups of consecutive whole
// requests rendered as one wavefront each, and each group's first-pass queue layout.
//
// A group holds at most `slots` sample items (a request larger than that forms a group of its own and
// regenerates its slots). Its first pass starts items item_lo .. item_lo + min(slots, items) - 1, queued
// request by request in item order: first the requests with spp >= min2 (walked in packets of two rays per
// lane), then those with spp >= min1 (one ray per lane), then the rest. queue_base[r] is the queue position,
// within its group, of request r's first item.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace spk {

struct BatchPlanGroup {
    uint64_t item_lo, item_hi;    // the group's sample items
    uint64_t packet_items;        // leading first-pass queue entries of requests with spp >= min1 (incl. min2)
    uint64_t packet2_items;       // leading first-pass queue entries of requests with spp >= min2
    uint32_t req_lo, req_hi;      // its requests
};

// items[r] = sample items of request r (pixels x spp); request r's items follow request r - 1's from 0.
inline std::vector<BatchPlanGroup> plan_batch(const uint64_t *items, const uint32_t *spp, uint32_t n, uint64_t slots,
                                              uint32_t min1, uint32_t min2, uint32_t *queue_base) {
    std::vector<BatchPlanGroup> groups;
    if (n == 0 || slots == 0) return groups;
    std::vector<uint64_t> base(n);
    uint64_t total = 0;
    for (uint32_t r = 0; r < n; ++r) {
        base[r] = total;
        total += items[r];
    }
    auto packet_class = [&](uint32_t r) { return spp[r] >= min2 ? 0 : spp[r] >= min1 ? 1 : 2; };
    auto close_group = [&](uint32_t r0, uint32_t r1) {
        const uint64_t lo = base[r0], hi = r1 < n ? base[r1] : total;
        const uint64_t first_end = lo + std::min<uint64_t>(slots, hi - lo);
        auto first_pass = [&](uint32_t r) {
            return std::min<uint64_t>(base[r] + items[r], first_end) - std::min<uint64_t>(base[r], first_end);
        };
        uint64_t class_items[3] = {0, 0, 0};
        for (uint32_t r = r0; r < r1; ++r) class_items[packet_class(r)] += first_pass(r);
        uint64_t pos[3] = {0, class_items[0], class_items[0] + class_items[1]};
        for (uint32_t r = r0; r < r1; ++r) {
            uint64_t &q = pos[packet_class(r)];
            queue_base[r] = static_cast<uint32_t>(q);
            q += first_pass(r);
        }
        groups.push_back(BatchPlanGroup{lo, hi, class_items[0] + class_items[1], class_items[0], r0, r1});
    };
    uint32_t r0 = 0;
    for (uint32_t r = 1; r < n; ++r) {
        if (base[r] + items[r] - base[r0] > slots) {
            close_group(r0, r);
            r0 = r;
        }
    }
    close_group(r0, n);
    return groups;
}

}  // namespace spk
