// heat1d_schedule.hpp -- placement of the 1-D groups on the warps of a one-CTA-per-SM launch.
//
// A group (32 equal-size instances, one warp) runs its whole time loop in one warp, and group
// costs differ by up to ~40x in a batch of uneven instances.  With one group per warp in
// blockIdx order the SMs that receive the costliest groups finish long after the others.  The
// factorised sweep launches one CTA per SM instead, and this placement balances the work of
// every SM sub-partition (warp w of a CTA runs on sub-partition w % 4): groups go, costliest
// first, to the least-loaded (SM, sub-partition) bin -- ties to the lowest bin, numbered
// sub-partition-major so that the first groups spread over all SMs -- and a bin's groups go,
// costliest first, to the least-loaded of its warps.  A warp runs its groups one after the other.
// Host-only (no CUDA): the CPU tests compile it directly.
#pragma once

#include <algorithm>
#include <functional>
#include <numeric>
#include <queue>
#include <utility>
#include <vector>

namespace lss_gb300 {
namespace heat1d {

constexpr int SUBPARTITIONS = 4; // warp schedulers per SM

struct warp_schedule {
    int ctas = 0;           // CTAs to launch (at most one per SM)
    int warps_per_cta = 0;
    std::vector<int> first; // per warp (ctas * warps_per_cta + 1 entries): start of its list in `group`
    std::vector<int> group; // group indices, warp after warp
};

// work[g]: cost of group g (points x time steps).  sms: SMs of the device; warps_per_cta: a
// multiple of SUBPARTITIONS.
inline warp_schedule schedule_groups(const std::vector<double> &work, int sms, int warps_per_cta)
{
    warp_schedule ws;
    ws.warps_per_cta = warps_per_cta;
    const int ng = static_cast<int>(work.size());
    if (ng == 0 || sms <= 0 || warps_per_cta < SUBPARTITIONS || warps_per_cta % SUBPARTITIONS) {
        ws.first.assign(1, 0);
        return ws;
    }
    std::vector<int> order(ng);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });

    // bins: sub-partition s of SM c is bin s * sms + c
    const int nbins = sms * SUBPARTITIONS;
    using item = std::pair<double, int>; // (load, index)
    std::priority_queue<item, std::vector<item>, std::greater<item>> heap;
    for (int b = 0; b < nbins; ++b) heap.push({0.0, b});
    std::vector<std::vector<int>> bin_groups(nbins);
    for (int g : order) {
        item top = heap.top();
        heap.pop();
        bin_groups[top.second].push_back(g);
        top.first += work[g];
        heap.push(top);
    }

    // warps of each bin: warp slot * SUBPARTITIONS + s of CTA c
    const int slots = warps_per_cta / SUBPARTITIONS;
    int ctas = 0;
    std::vector<std::vector<int>> warp_groups(static_cast<size_t>(sms) * warps_per_cta);
    for (int b = 0; b < nbins; ++b) {
        if (bin_groups[b].empty()) continue;
        const int s = b / sms, c = b % sms;
        ctas = std::max(ctas, c + 1);
        std::priority_queue<item, std::vector<item>, std::greater<item>> wh;
        for (int j = 0; j < slots; ++j) wh.push({0.0, j});
        for (int g : bin_groups[b]) { // already costliest first
            item top = wh.top();
            wh.pop();
            warp_groups[static_cast<size_t>(c) * warps_per_cta + top.second * SUBPARTITIONS + s].push_back(g);
            top.first += work[g];
            wh.push(top);
        }
    }
    ws.ctas = ctas;
    const size_t nw = static_cast<size_t>(ctas) * warps_per_cta;
    ws.first.assign(nw + 1, 0);
    ws.group.reserve(ng);
    for (size_t w = 0; w < nw; ++w) {
        ws.first[w] = static_cast<int>(ws.group.size());
        ws.group.insert(ws.group.end(), warp_groups[w].begin(), warp_groups[w].end());
    }
    ws.first[nw] = static_cast<int>(ws.group.size());
    return ws;
}

} // namespace heat1d
} // namespace lss_gb300
