// Launch items for a captured contraction: which steps share one grouped
// launch (jetgpu_contract_group) and in what order the items run. Used by
// the TaskBasedContractor's replay and by the SlicedContractor's chunk graph.
//
// Steps come in a dependency order (every input is a leaf or the output of
// an earlier step). Consecutive steps that may be grouped (tiny products)
// form a run, which a step that may not be grouped ends. Within a run the
// steps are scheduled by level -- level 0 reads nothing the run produces,
// level l reads some output of level l - 1 and none of a later level -- and
// each level becomes one item (or several of at most `max_group` steps),
// lowest level first. Steps outside runs keep their own items, in order. A circuit network whose tiny steps form
// chains that interleave (a 16-qubit, 8-cycle random circuit: 206 of its 207
// path steps tiny) needs 17 items this way, against 91 when a run stops at
// the first step that reads the run's own output.
//
// Every step's inputs are produced by an earlier item, and no item reads
// its own outputs; liveness plans must go by item position, since steps of
// one run no longer run in step order.
#pragma once

#include <algorithm>
#include <array>
#include <cstddef>
#include <unordered_map>
#include <vector>

namespace Jet {
namespace group_schedule {

// groupable[i]: step i may share a launch; inputs[i]: its two input ids;
// outputs[i]: its output id (ids shared with the inputs'). Returns the items,
// each a list of step indices.
inline std::vector<std::vector<size_t>> Items(const std::vector<char> &groupable,
                                              const std::vector<std::array<size_t, 2>> &inputs,
                                              const std::vector<size_t> &outputs,
                                              size_t max_group)
{
    std::vector<std::vector<size_t>> items;
    std::vector<size_t> run;
    auto flush = [&] {
        if (run.empty())
            return;
        std::unordered_map<size_t, size_t> level_of; // run output -> level
        std::vector<size_t> level(run.size());
        size_t top = 0;
        for (size_t r = 0; r < run.size(); ++r) {
            size_t l = 0;
            for (size_t in : inputs[run[r]]) {
                const auto it = level_of.find(in);
                if (it != level_of.end())
                    l = std::max(l, it->second + 1);
            }
            level[r] = l;
            level_of[outputs[run[r]]] = l;
            top = std::max(top, l);
        }
        for (size_t l = 0; l <= top; ++l) {
            std::vector<size_t> item;
            for (size_t r = 0; r < run.size(); ++r) {
                if (level[r] != l)
                    continue;
                if (item.size() == max_group) {
                    items.push_back(std::move(item));
                    item.clear();
                }
                item.push_back(run[r]);
            }
            if (!item.empty())
                items.push_back(std::move(item));
        }
        run.clear();
    };
    for (size_t i = 0; i < groupable.size(); ++i) {
        if (groupable[i]) {
            run.push_back(i);
            continue;
        }
        flush();
        items.push_back({i});
    }
    flush();
    return items;
}

} // namespace group_schedule
} // namespace Jet
