// Splitting one batch of independent systems over several GPUs (or ranks):
// gbdpcg_partition.  The systems share nothing, so the only decision is who
// solves which; there is no exchange of data while they are solved, and the
// caller gathers the per-system results afterwards.  The split balances the
// estimated cost of each part: a system costs about n^2 N per PCG iteration
// (its block rows, include/pcg.cuh:157-184) times its iterations.  The greedy
// longest-processing-time rule places the systems in decreasing cost, each on
// the part with the least cost so far (ties: the lowest part index), which
// keeps every part within 4/3 of the optimum and, on batches of many small
// systems, within a fraction of one system's cost of the mean.
// Host code only: no CUDA call.
#include <stdint.h>

#include <algorithm>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "../../include/gbdpcg.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

extern "C" {

int gbdpcg_partition(const uint32_t *n, const uint32_t *N, const float *iters, uint32_t count, uint32_t parts,
                     uint32_t *part_of, double *part_cost) {
    if (!n || !N || !part_of || count == 0 || parts == 0) {
        gbdpcg::set_last_error("NULL pointer, empty batch or no parts");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    std::vector<double> cost(count);
    for (uint32_t i = 0; i < count; ++i) {
        const double it = iters ? (double)iters[i] : 1.0;
        if (n[i] == 0 || N[i] == 0 || !(it > 0)) {
            gbdpcg::set_last_error("system " + std::to_string(i) + ": sizes and iterations must be positive");
            return GBDPCG_ERR_INVALID_ARGUMENT;
        }
        cost[i] = (double)n[i] * n[i] * N[i] * it;
    }
    std::vector<uint32_t> order(count);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
    // min-heap of (load, part)
    using Slot = std::pair<double, uint32_t>;
    std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
    for (uint32_t p = 0; p < parts; ++p) heap.push({0.0, p});
    std::vector<double> load(parts, 0.0);
    for (uint32_t i : order) {
        const Slot s = heap.top();
        heap.pop();
        part_of[i] = s.second;
        load[s.second] = s.first + cost[i];
        heap.push({load[s.second], s.second});
    }
    if (part_cost)
        for (uint32_t p = 0; p < parts; ++p) part_cost[p] = load[p];
    return GBDPCG_SUCCESS;
}

}  // extern "C"
