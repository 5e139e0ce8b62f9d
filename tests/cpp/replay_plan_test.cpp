// Host-side check of the TaskBasedContractor replay's scheduling
// (jet_gb300/include/jet/TaskBasedContractor.hpp, Jet::replay_detail): on
// random contraction DAGs (steps reading leaves or earlier outputs, tiny and
// large shapes mixed),
//  * GroupTinySteps keeps step order, puts only tiny steps (m n k below the
//    limit, k <= 64) in runs, never a step that reads its run's own outputs,
//    at most 256 per run, and nothing in runs when grouping is off;
//  * PlanArena never lets two buffers that are live at the same time overlap:
//    an output is live from its item to the item of its last consumer (to
//    the end when nothing reads it), and a run's outputs are all live while
//    the run executes.
// No GPU is used.
#include "Jet.hpp"

#include <cstdio>
#include <random>
#include <vector>

using namespace Jet::replay_detail;

#define FAIL(...)                                                                                  \
    do {                                                                                           \
        std::printf(__VA_ARGS__);                                                                  \
        return 1;                                                                                  \
    } while (0)

int Check(std::mt19937 &rng, int trial)
{
    const size_t n_leaves = 2 + rng() % 400, n_steps = 1 + rng() % 400;
    std::vector<StepShape> steps;
    std::vector<int> leaf_of(n_leaves);
    for (size_t i = 0; i < n_leaves; ++i)
        leaf_of[i] = (int)i;
    std::vector<size_t> avail;
    for (size_t i = 0; i < n_leaves; ++i)
        avail.push_back(i);
    std::vector<size_t> bytes(n_leaves, 0);
    for (size_t s = 0; s < n_steps && avail.size() >= 2; ++s) {
        // Operands: two distinct available buffers (consumed, as in a path).
        const size_t ia = rng() % avail.size();
        const size_t a = avail[ia];
        avail.erase(avail.begin() + ia);
        const size_t ib = rng() % avail.size();
        const size_t b = avail[ib];
        avail.erase(avail.begin() + ib);
        const size_t out = leaf_of.size();
        leaf_of.push_back(-1);
        const bool big = rng() % 5 == 0;
        const uint64_t m = big ? 1 + rng() % 4096 : 1 + rng() % 64;
        const uint64_t n = big ? 1 + rng() % 4096 : 1 + rng() % 64;
        const uint64_t k = big ? 1 + rng() % 512 : 1 + rng() % 80;
        bytes.push_back(std::max<uint64_t>(m * n, 1) * 8);
        steps.push_back({a, b, out, m, n, k});
        avail.push_back(out);
    }
    const double max_work = 131072.0;
    for (bool enabled : {true, false}) {
        const auto items = GroupTinySteps(steps, enabled, max_work);
        size_t next = 0;
        for (const auto &item : items) {
            if (item.empty() || item.size() > 256)
                FAIL("trial %d: item of %zu steps\n", trial, item.size());
            std::vector<size_t> outs;
            for (size_t i : item) {
                if (i != next++)
                    FAIL("trial %d: steps out of order\n", trial);
                const StepShape &st = steps[i];
                const bool tiny =
                    st.k <= 64 && (double)st.m * (double)st.n * (double)st.k < max_work;
                if (item.size() > 1 && (!tiny || !enabled))
                    FAIL("trial %d: step %zu grouped but not tiny or grouping off\n", trial, i);
                for (size_t o : outs)
                    if (st.a == o || st.b == o)
                        FAIL("trial %d: step %zu reads its run's output\n", trial, i);
                outs.push_back(st.out);
            }
        }
        if (next != steps.size())
            FAIL("trial %d: %zu of %zu steps scheduled\n", trial, next, steps.size());
        std::vector<size_t> offset;
        const size_t top = PlanArena(steps, items, leaf_of, bytes, offset);
        // Lifetimes in items: first = the producing item, end = the consuming item.
        std::vector<size_t> item_of(steps.size());
        for (size_t t = 0; t < items.size(); ++t)
            for (size_t i : items[t])
                item_of[i] = t;
        std::vector<long> first(leaf_of.size(), -1), end(leaf_of.size(), -1);
        for (size_t i = 0; i < steps.size(); ++i) {
            first[steps[i].out] = (long)item_of[i];
            end[steps[i].out] = (long)items.size(); // until read (or to the end)
        }
        std::vector<int> read(leaf_of.size(), 0);
        for (size_t i = 0; i < steps.size(); ++i)
            for (size_t in : {steps[i].a, steps[i].b})
                if (leaf_of[in] < 0) {
                    end[in] = (long)item_of[i];
                    read[in] = 1;
                }
        for (size_t x = 0; x < leaf_of.size(); ++x) {
            if (leaf_of[x] >= 0)
                continue;
            if (offset[x] % 256 || offset[x] + bytes[x] > top)
                FAIL("trial %d: buffer %zu outside the arena\n", trial, x);
            for (size_t y = x + 1; y < leaf_of.size(); ++y) {
                if (leaf_of[y] >= 0)
                    continue;
                // Both live during some item (inclusive ranges).
                if (first[x] > end[y] || first[y] > end[x])
                    continue;
                const bool apart = offset[x] + bytes[x] <= offset[y] ||
                                   offset[y] + bytes[y] <= offset[x];
                if (!apart)
                    FAIL("trial %d (grouping %d): buffers %zu [%ld, %ld] and %zu [%ld, %ld] "
                         "overlap\n",
                         trial, enabled, x, first[x], end[x], y, first[y], end[y]);
            }
        }
    }
    return 0;
}

int main()
{
    std::mt19937 rng(20240601);
    for (int trial = 0; trial < 300; ++trial)
        if (Check(rng, trial))
            return 1;
    std::printf("ok 300 plans\n");
    return 0;
}
