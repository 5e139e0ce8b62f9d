// Host-side check of the TaskBasedContractor replay's scheduling
// (jet_gb300/include/jet/TaskBasedContractor.hpp, Jet::replay_detail): on
// random contraction DAGs (steps reading leaves or earlier outputs, tiny and
// large shapes mixed),
//  * GroupTinySteps schedules every step once, after the items that produce
//    its inputs; puts only tiny steps (m n k below the limit, k <= 64) in
//    items of several steps, never a step that reads its item's own outputs,
//    at most 256 per item; keeps steps that are not tiny in step order with
//    every run of tiny steps between the same two of them; and keeps plain
//    step order, one step per item, when grouping is off;
//  * PlanArena never lets two buffers that are live at the same time overlap:
//    an output is live from its item to the last item that reads it (to the
//    end when nothing reads it), and an item's outputs are all live while
//    the item executes.
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

int Verify(const std::vector<StepShape> &steps, const std::vector<int> &leaf_of,
           const std::vector<size_t> &bytes, int trial);

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
        // Operands: two distinct available buffers, consumed as in a path,
        // except that one in six first operands stays available for a later
        // step too (a subtree shared by two networks of one contractor).
        const size_t ia = rng() % avail.size();
        const size_t a = avail[ia];
        if (rng() % 6 != 0)
            avail.erase(avail.begin() + ia);
        else
            std::swap(avail[ia], avail.back()); // b is drawn from the others
        const size_t n_other = avail.size() - (avail.back() == a ? 1 : 0);
        if (n_other == 0)
            break;
        const size_t ib = rng() % n_other;
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
    return Verify(steps, leaf_of, bytes, trial);
}

int Verify(const std::vector<StepShape> &steps, const std::vector<int> &leaf_of,
           const std::vector<size_t> &bytes, int trial)
{
    const double max_work = 131072.0;
    auto is_tiny = [&](const StepShape &st) {
        return st.k <= 64 && (double)st.m * (double)st.n * (double)st.k < max_work;
    };
    std::vector<long> producer(leaf_of.size(), -1); // step producing each buffer
    for (size_t i = 0; i < steps.size(); ++i)
        producer[steps[i].out] = (long)i;
    for (bool enabled : {true, false}) {
        const auto items = GroupTinySteps(steps, enabled, max_work);
        std::vector<long> item_of_step(steps.size(), -1);
        for (size_t t = 0; t < items.size(); ++t) {
            const auto &item = items[t];
            if (item.empty() || item.size() > 256)
                FAIL("trial %d: item of %zu steps\n", trial, item.size());
            for (size_t i : item) {
                if (i >= steps.size() || item_of_step[i] >= 0)
                    FAIL("trial %d: step %zu scheduled twice\n", trial, i);
                item_of_step[i] = (long)t;
                if (item.size() > 1 && (!is_tiny(steps[i]) || !enabled))
                    FAIL("trial %d: step %zu grouped but not tiny or grouping off\n", trial, i);
            }
        }
        size_t last_big = 0;
        long last_big_item = -1;
        for (size_t i = 0; i < steps.size(); ++i) {
            const long t = item_of_step[i];
            if (t < 0)
                FAIL("trial %d: step %zu not scheduled\n", trial, i);
            for (size_t in : {steps[i].a, steps[i].b})
                if (producer[in] >= 0 && item_of_step[producer[in]] >= t)
                    FAIL("trial %d: step %zu runs before or with the step it reads\n", trial, i);
            if (!enabled && t != (long)i)
                FAIL("trial %d: grouping off, step %zu in item %ld\n", trial, i, t);
            if (enabled && !is_tiny(steps[i])) {
                // Non-tiny steps in order, and the tiny steps before this one
                // (since the previous non-tiny step) in items between the two.
                if (t <= last_big_item)
                    FAIL("trial %d: step %zu out of order\n", trial, i);
                for (size_t j = last_big; j < i; ++j)
                    if (item_of_step[j] <= last_big_item || item_of_step[j] >= t)
                        FAIL("trial %d: tiny step %zu leaves its run\n", trial, j);
                last_big = i + 1;
                last_big_item = t;
            }
        }
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
                    end[in] = read[in] ? std::max(end[in], (long)item_of[i]) : (long)item_of[i];
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

// A buffer read by two tiny steps of one run where the later step (in step
// order) runs in the earlier level: its lifetime must end with the other.
int SharedAcrossLevels()
{
    std::vector<int> leaf_of = {0, 1, 2, 3};
    std::vector<size_t> bytes = {0, 0, 0, 0};
    std::vector<StepShape> steps;
    auto add = [&](size_t a, size_t b, uint64_t m, uint64_t n, uint64_t k) {
        steps.push_back({a, b, leaf_of.size(), m, n, k});
        leaf_of.push_back(-1);
        bytes.push_back(std::max<uint64_t>(m * n, 1) * 8);
        return leaf_of.size() - 1;
    };
    const size_t x = add(0, 1, 4096, 4096, 256); // not tiny: X = 4
    const size_t y = add(2, 3, 4, 4, 4);         // level 0
    add(y, x, 4, 4, 4);                          // level 1, reads X
    add(x, 3, 8, 8, 4);                          // level 0, reads X too
    return Verify(steps, leaf_of, bytes, -1);
}

int main()
{
    if (SharedAcrossLevels())
        return 1;
    std::mt19937 rng(20240601);
    for (int trial = 0; trial < 300; ++trial)
        if (Check(rng, trial))
            return 1;
    std::printf("ok 300 plans\n");
    return 0;
}
