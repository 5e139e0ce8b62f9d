// Jet::TaskBasedContractor on a GB300 (reference:
// include/jet/TaskBasedContractor.hpp).
//
// The reference turns every path step of every added network into a Taskflow
// task ("<step id>:<step name>", with ":results[i]" on a network's final
// step), shares tasks whose names coincide across networks (the
// slice-independent subtrees of a sliced network), adds storage, deletion and
// reduction tasks and runs the DAG on a thread pool.
//
// Here the same bookkeeping (names, sharing, parents, flop and memory
// counters, result slots) drives a single stream-ordered schedule: Contract()
// walks the tasks in dependency order on one host thread and enqueues each
// contraction on the library CUDA stream -- the GPU pipelines the kernels,
// with no host synchronisation between steps. Intermediates are released to
// the stream-ordered allocator as soon as their last consumer is enqueued
// (the deletion tasks), so peak device memory follows the path's liveness.
// The reduction of equal-shaped results runs as an FP64 sum on the device.
//
// Repeated Contract() calls of the same tasks replay a CUDA graph: the first
// call runs the tasks eagerly as above (keeping a copy of every leaf), the
// second captures the contractions and result copies into one graph over an
// arena planned from the tasks' liveness (PathInfo's step sizes), and that
// call and every later one launch the graph, with no per-task host work.
#pragma once

#include <algorithm>
#include <array>
#include <future>
#include <map>
#include <memory>
#include <ostream>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "GroupSchedule.hpp"
#include "PathInfo.hpp"
#include "Tensor.hpp"
#include "TensorNetwork.hpp"

namespace Jet {

// The replay plan's scheduling, kept apart from the contractor so that it
// can be checked without a GPU (tests/cpp/replay_plan_test.cpp).
namespace replay_detail {

// One contraction step: operand and output buffer ids, product shape.
struct StepShape {
    size_t a, b, out;
    uint64_t m, n, k;
};

// Launch items: one step, or (when `enabled`) a level of a run of tiny steps
// -- m n k below `max_work` and k <= 64 -- none of which reads another's
// output, at most 256 per item (a grouped launch's task limit); see
// group_schedule::Items for the order.
inline std::vector<std::vector<size_t>> GroupTinySteps(const std::vector<StepShape> &steps,
                                                       bool enabled, double max_work)
{
    std::vector<char> groupable(steps.size());
    std::vector<std::array<size_t, 2>> inputs(steps.size());
    std::vector<size_t> outputs(steps.size());
    for (size_t i = 0; i < steps.size(); ++i) {
        const StepShape &st = steps[i];
        groupable[i] = enabled && st.k <= 64 &&
                       (double)st.m * (double)st.n * (double)st.k < max_work;
        inputs[i] = {st.a, st.b};
        outputs[i] = st.out;
    }
    return group_schedule::Items(groupable, inputs, outputs, 256);
}

// First-fit arena offsets (256-byte aligned) of every step output, over its
// lifetime: from its item to the last item that reads it (never, for an
// output no step reads). An item's outputs are all allocated before any input
// it reads for the last time is released: a grouped launch runs its steps
// together. Leaves (leaf_of >= 0) live outside the arena. Returns the arena's
// size; offset[b] is set for every step output b.
inline size_t PlanArena(const std::vector<StepShape> &steps,
                        const std::vector<std::vector<size_t>> &items,
                        const std::vector<int> &leaf_of, const std::vector<size_t> &bytes,
                        std::vector<size_t> &offset)
{
    const size_t nb = leaf_of.size();
    std::vector<long> last(nb, -1); // the last item reading each buffer
    for (size_t t = 0; t < items.size(); ++t)
        for (size_t i : items[t]) {
            last[steps[i].a] = std::max(last[steps[i].a], (long)t);
            last[steps[i].b] = std::max(last[steps[i].b], (long)t);
        }
    offset.assign(nb, 0);
    std::map<size_t, size_t> free_blocks;
    size_t top = 0;
    auto alloc = [&](size_t n) {
        n = (n + 255) / 256 * 256;
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it)
            if (it->second >= n) {
                const size_t off = it->first, rem = it->second - n;
                free_blocks.erase(it);
                if (rem)
                    free_blocks[off + n] = rem;
                return off;
            }
        top += n;
        return top - n;
    };
    auto release = [&](size_t off, size_t n) {
        n = (n + 255) / 256 * 256;
        auto it = free_blocks.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_blocks.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_blocks.erase(nx);
        }
        if (it != free_blocks.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_blocks.erase(it);
            }
        }
    };
    for (size_t t = 0; t < items.size(); ++t) {
        for (size_t i : items[t])
            offset[steps[i].out] = alloc(bytes[steps[i].out]);
        for (size_t i : items[t])
            for (size_t in : {steps[i].a, steps[i].b})
                if (leaf_of[in] < 0 && last[in] == (long)t) {
                    release(offset[in], bytes[in]);
                    last[in] = -2; // released once
                }
    }
    return top;
}

} // namespace replay_detail

template <class TensorType> class TaskBasedContractor {
  public:
    struct Task {
        enum Kind { CONTRACT, STORE, DELETE, REDUCE } kind;
        std::string name;
        std::string input_1, input_2;
        size_t result_id;
    };

    using NameToTaskMap = std::unordered_map<std::string, size_t>;
    using NameToTensorMap = std::unordered_map<std::string, std::unique_ptr<TensorType>>;
    using NameToParentsMap = std::unordered_map<std::string, std::unordered_set<std::string>>;

    explicit TaskBasedContractor(size_t num_threads = std::thread::hardware_concurrency())
        : num_threads_(num_threads)
    {
    }

    const NameToTaskMap &GetNameToTaskMap() const noexcept { return name_to_task_; }
    const NameToTensorMap &GetNameToTensorMap() const noexcept { return name_to_tensor_; }
    const NameToParentsMap &GetNameToParentsMap() const noexcept { return name_to_parents_; }
    const std::vector<TensorType> &GetResults() const noexcept { return results_; }
    const TensorType &GetReductionResult() const noexcept { return reduction_result_; }
    const std::vector<Task> &GetTasks() const noexcept { return tasks_; }
    double GetFlops() const noexcept { return flops_; }
    double GetMemory() const noexcept { return memory_; }

    // Adds the steps of `tn` along `path_info`; returns how many of them were
    // already present under the same name (shared with an earlier network).
    size_t AddContractionTasks(const TensorNetwork<TensorType> &tn,
                               const PathInfo &path_info) noexcept
    {
        const auto &path = path_info.GetPath();
        const auto &steps = path_info.GetSteps();
        if (path.empty())
            return 0;
        ResetReplay();
        const auto &nodes = tn.GetNodes();
        const size_t num_leaves = nodes.size();
        const size_t result_id = results_.size();
        results_.resize(result_id + 1);
        size_t shared = 0;
        // The contractor's own copy of each leaf, taken once per name. On the
        // GPU it is made device resident here, as the reference's CudaTensor
        // leaves are when the tasks are added, so that Contract() runs only
        // the contraction; the uploads end before this call returns. A copy
        // that cannot be uploaded now (device memory exhausted) stays on the
        // host and is uploaded at its first use, whose failure Contract()
        // reports.
        bool uploaded = false;
        auto take_leaf = [&](const std::string &name, size_t id) {
            if (name_to_tensor_.count(name))
                return;
            auto copy = std::make_unique<TensorType>(nodes[id].tensor);
            if constexpr (kGpuTensor) {
                try {
                    copy->GetDeviceData();
                    uploaded = true;
                } catch (const Exception &) {
                }
            }
            name_to_tensor_.emplace(name, std::move(copy));
        };
        for (size_t i = 0; i < path.size(); ++i) {
            const auto [id_1, id_2] = path[i];
            const std::string name_1 = TaskName(steps[id_1]);
            const std::string name_2 = TaskName(steps[id_2]);
            std::string name_3 = TaskName(steps[num_leaves + i]);
            const bool last = i + 1 == path.size();
            if (last)
                name_3 += ":results[" + std::to_string(result_id) + "]";
            name_to_parents_[name_1].insert(name_3);
            name_to_parents_[name_2].insert(name_3);
            if (id_1 < num_leaves)
                take_leaf(name_1, id_1);
            if (id_2 < num_leaves)
                take_leaf(name_2, id_2);
            name_to_tensor_.try_emplace(name_3, nullptr);
            if (name_to_task_.count(name_3)) {
                ++shared;
                continue;
            }
            flops_ += path_info.GetPathStepFlops(steps[num_leaves + i].id);
            memory_ += path_info.GetPathStepMemory(steps[num_leaves + i].id);
            name_to_task_.emplace(name_3, tasks_.size());
            tasks_.push_back(Task{Task::CONTRACT, name_3, name_1, name_2, 0});
            if (last)
                tasks_.push_back(Task{Task::STORE, name_3, "", "", result_id});
        }
        if constexpr (kGpuTensor) {
            if (uploaded) {
                try {
                    Gpu::Synchronize();
                } catch (const Exception &) { // reported by the next device call
                }
            }
        }
        return shared;
    }

    size_t AddReductionTask() noexcept
    {
        ResetReplay();
        if (reduced_)
            return 0;
        reduced_ = true;
        tasks_.push_back(Task{Task::REDUCE, "reduce", "", "", 0});
        return 1;
    }

    size_t AddDeletionTasks() noexcept
    {
        ResetReplay();
        size_t count = 0;
        for (const auto &kv : name_to_parents_) {
            if (kv.second.empty())
                continue;
            tasks_.push_back(Task{Task::DELETE, kv.first + ":delete", kv.first, "", 0});
            ++count;
        }
        return count;
    }

    // Runs every task; the future is ready once the device work is complete.
    std::future<void> Contract()
    {
        return std::async(std::launch::async, [this] {
            if (!Replayable())
                Run();
            else if (runs_ == 0)
                RunAndKeepLeaves();
            else
                Replay();
            ++runs_;
        });
    }

    // Graph replay of repeated Contract() calls (default on); off: every call
    // runs the tasks eagerly.
    void SetGraphReplay(bool on)
    {
        replay_on_ = on;
        ResetReplay();
    }
    // Grouped launches of independent tiny steps in the replayed graph
    // (default on; off: one launch per step, as the eager run).
    void SetGrouping(bool on)
    {
        grouping_ = on;
        ResetReplay();
    }
    // Whether the next Contract() launches a captured graph.
    bool HasReplayGraph() const noexcept { return replay_.graph != nullptr; }

    ~TaskBasedContractor() { ResetReplay(); }

  private:
    // The replay runs on this package's Jet::Tensor; for other tensor types
    // (CudaTensor) Contract() stays eager and S only names a valid type.
    static constexpr bool kGpuTensor =
        std::is_same_v<TensorType, Tensor<std::complex<float>>> ||
        std::is_same_v<TensorType, Tensor<std::complex<double>>>;
    using S = std::conditional_t<kGpuTensor, typename TensorType::scalar_type_t,
                                 std::complex<float>>;

    // What the captured graph reads and writes: leaf copies, one arena for
    // the intermediates (first-fit over their lifetimes), the largest step's
    // workspace, and per contraction task its operands' buffers and layout.
    struct ReplayPlan {
        struct Step {
            size_t a, b, out;
            typename Tensor<S>::ContractionLayout layout;
        };
        // By leaf slot: the leaves the tasks read, taken over from the first
        // run as its deletion tasks release them (owned), else still held by
        // the contractor (leaves points there).
        std::vector<std::unique_ptr<Tensor<S>>> owned;
        std::vector<const Tensor<S> *> leaves;
        std::unordered_map<std::string, size_t> leaf_slot;
        std::vector<Step> steps;
        std::vector<size_t> offset, bytes;         // per buffer id
        std::vector<int> leaf_of;                  // per buffer id: leaf slot or -1
        std::vector<std::pair<size_t, size_t>> stores; // (buffer id, result index)
        Gpu::DeviceBuffer arena, ws;
        Gpu::DeviceBuffer groups; // task tables of the grouped tiny steps
        int precision = -1;
        void *graph = nullptr;
    };
    ReplayPlan replay_;
    bool replay_on_ = true;
    bool grouping_ = true;
    // Steps whose batch m n k is below this replay in grouped launches.
    static constexpr double kGroupMaxWork = 131072.0;

    // Number of leading axes of `perm` whose dimensions multiply to `extent`.
    static size_t SplitCount(const std::vector<uint64_t> &shape, const std::vector<int32_t> &perm,
                             uint64_t extent)
    {
        size_t j = 0;
        uint64_t p = 1;
        while (j < perm.size() && p < extent)
            p *= shape[perm[j++]];
        return j;
    }

    // Appends the element offsets of every index over axes perm[from..to)
    // (row-major, the last fastest) of a row-major tensor; returns where
    // they start.
    static size_t AppendOffsets(std::vector<int64_t> &out, const std::vector<uint64_t> &shape,
                                const std::vector<int32_t> &perm, size_t from, size_t to)
    {
        std::vector<int64_t> st(shape.size(), 1);
        for (int i = (int)shape.size() - 2; i >= 0; --i)
            st[i] = st[i + 1] * (int64_t)shape[i + 1];
        uint64_t count = 1;
        for (size_t j = from; j < to; ++j)
            count *= shape[perm[j]];
        const size_t at = out.size();
        for (uint64_t idx = 0; idx < count; ++idx) {
            uint64_t x = idx;
            int64_t off = 0;
            for (size_t j = to; j-- > from;) {
                const int a = perm[j];
                off += (int64_t)(x % shape[a]) * st[a];
                x /= shape[a];
            }
            out.push_back(off);
        }
        return at;
    }
    bool keep_leaves_ = false; // Run() hands released leaves to replay_
    size_t runs_ = 0;

    bool Replayable() const noexcept { return kGpuTensor && replay_on_; }

    void ResetReplay() noexcept
    {
        if (replay_.graph != nullptr)
            jetgpu_graph_destroy(replay_.graph);
        replay_ = ReplayPlan();
        runs_ = 0;
    }

    // First run: the eager schedule, keeping every leaf the tasks read for
    // the replays (the deletion tasks would release the contractor's own
    // leaves; they are handed over instead, without a copy).
    void RunAndKeepLeaves()
    {
        if constexpr (kGpuTensor) {
            std::unordered_set<std::string> produced;
            for (const Task &t : tasks_)
                if (t.kind == Task::CONTRACT)
                    produced.insert(t.name);
            std::vector<const std::string *> names;
            for (const Task &t : tasks_) {
                if (t.kind != Task::CONTRACT)
                    continue;
                for (const std::string *in : {&t.input_1, &t.input_2})
                    if (!produced.count(*in) && !replay_.leaf_slot.count(*in)) {
                        replay_.leaf_slot.emplace(*in, names.size());
                        names.push_back(in);
                    }
            }
            replay_.owned.resize(names.size());
            replay_.leaves.assign(names.size(), nullptr);
            replay_.precision = Tensor<S>::template ContractPrecision<S>();
            keep_leaves_ = true;
            try {
                Run();
            } catch (...) {
                keep_leaves_ = false;
                throw;
            }
            keep_leaves_ = false;
            for (size_t i = 0; i < names.size(); ++i)
                replay_.leaves[i] = replay_.owned[i] ? replay_.owned[i].get()
                                                     : name_to_tensor_.at(*names[i]).get();
        }
        else {
            Run();
        }
    }

    void Replay()
    {
        if constexpr (kGpuTensor) {
            Gpu::Range range("Jet::TaskBasedContractor::Contract (graph)");
            if (replay_.graph != nullptr &&
                replay_.precision != Tensor<S>::template ContractPrecision<S>()) {
                jetgpu_graph_destroy(replay_.graph);
                replay_.graph = nullptr;
                replay_.precision = Tensor<S>::template ContractPrecision<S>();
            }
            if (replay_.graph == nullptr)
                Capture();
            Gpu::Check(jetgpu_graph_launch(replay_.graph, Gpu::Stream()), "graph launch");
            for (const auto &st : replay_.stores)
                results_[st.second].GetMutableDeviceData(); // the host copy is stale
            for (const Task &task : tasks_)
                if (task.kind == Task::REDUCE)
                    Reduce();
            Gpu::Synchronize();
        }
    }

    void Capture()
    {
        if constexpr (kGpuTensor) {
            ReplayPlan &r = replay_;
            r.steps.clear();
            r.stores.clear();
            std::unordered_map<std::string, size_t> id;
            std::vector<Tensor<S>> shape_of; // per buffer id: labels and shape, no data
            auto buffer = [&](const std::string &name) -> size_t {
                const auto it = id.find(name);
                if (it != id.end())
                    return it->second;
                const auto leaf = r.leaf_slot.at(name);
                id.emplace(name, shape_of.size());
                shape_of.push_back(
                    Tensor<S>(r.leaves[leaf]->GetIndices(), r.leaves[leaf]->GetShape()));
                r.leaf_of.push_back((int)leaf);
                return shape_of.size() - 1;
            };
            const int dt = Gpu::DtypeCode<S>();
            size_t ws = 0;
            for (const Task &t : tasks_) {
                if (t.kind == Task::CONTRACT) {
                    const size_t a = buffer(t.input_1);
                    const size_t b = buffer(t.input_2);
                    auto layout = Tensor<S>::template LayoutOf<S>(shape_of[a], shape_of[b]);
                    const auto &l = layout;
                    ws = std::max(ws, jetgpu_contract_workspace_size(
                                          (int)l.a_shape.size(), l.a_shape.data(), l.a_perm.data(),
                                          (int)l.b_shape.size(), l.b_shape.data(), l.b_perm.data(),
                                          l.m, l.n, l.k, dt, r.precision));
                    id[t.name] = shape_of.size();
                    shape_of.push_back(Tensor<S>(l.c_indices, l.c_shape));
                    r.leaf_of.push_back(-1);
                    r.steps.push_back({a, b, shape_of.size() - 1, std::move(layout)});
                }
                else if (t.kind == Task::STORE) {
                    r.stores.emplace_back(id.at(t.name), t.result_id);
                }
            }
            // Launch items (single steps, or runs of independent tiny steps
            // replayed as one grouped launch) and the arena offsets of the
            // intermediates over their lifetimes (replay_detail below).
            const size_t nb = shape_of.size();
            std::vector<replay_detail::StepShape> shapes(r.steps.size());
            for (size_t i = 0; i < r.steps.size(); ++i) {
                const auto &st = r.steps[i];
                shapes[i] = {st.a, st.b, st.out, st.layout.m, st.layout.n, st.layout.k};
            }
            const bool plain =
                r.precision == JETGPU_PREC_FP32 || r.precision == JETGPU_PREC_AUTO;
            const std::vector<std::vector<size_t>> items =
                replay_detail::GroupTinySteps(shapes, grouping_ && plain, kGroupMaxWork);
            r.bytes.assign(nb, 0);
            for (const auto &st : r.steps)
                r.bytes[st.out] = std::max<size_t>(shape_of[st.out].GetSize(), 1) * sizeof(S);
            const size_t top =
                replay_detail::PlanArena(shapes, items, r.leaf_of, r.bytes, r.offset);
            r.arena = Gpu::DeviceBuffer(std::max<size_t>(top, 256));
            r.ws = Gpu::DeviceBuffer(ws);
            auto ptr = [&](size_t b) -> void * {
                if (r.leaf_of[b] >= 0)
                    return const_cast<S *>(r.leaves[r.leaf_of[b]]->GetDeviceData());
                return static_cast<char *>(r.arena.get()) + r.offset[b];
            };
            // Leaf and result buffers are resolved (and, if need be, uploaded)
            // before the capture: nothing below may allocate or copy from host.
            for (size_t b = 0; b < nb; ++b)
                if (r.leaf_of[b] >= 0)
                    ptr(b);
            std::vector<void *> result_ptr(r.stores.size());
            for (size_t i = 0; i < r.stores.size(); ++i)
                result_ptr[i] = results_[r.stores[i].second].GetMutableDeviceData();
            // Task tables of the grouped items: per task the element offsets
            // of A's rows and columns and of B's, in the product's view
            // (left ++ common of A, common ++ right of B), and one batch offset.
            std::vector<int64_t> tables{0}; // entry 0: the batch offset
            std::vector<std::array<size_t, 4>> table_at(r.steps.size());
            size_t n_tasks = 0;
            for (const auto &item : items) {
                if (item.size() < 2)
                    continue;
                for (size_t i : item) {
                    const auto &l = r.steps[i].layout;
                    const size_t na = SplitCount(l.a_shape, l.a_perm, l.m);
                    const size_t nb_ = SplitCount(l.b_shape, l.b_perm, l.k);
                    table_at[i] = {AppendOffsets(tables, l.a_shape, l.a_perm, 0, na),
                                   AppendOffsets(tables, l.a_shape, l.a_perm, na,
                                                 l.a_perm.size()),
                                   AppendOffsets(tables, l.b_shape, l.b_perm, 0, nb_),
                                   AppendOffsets(tables, l.b_shape, l.b_perm, nb_,
                                                 l.b_perm.size())};
                    ++n_tasks;
                }
            }
            const size_t tables_bytes = (tables.size() * sizeof(int64_t) + 255) / 256 * 256;
            r.groups = Gpu::DeviceBuffer(n_tasks ? tables_bytes + n_tasks * sizeof(jetgpu_group_task)
                                                 : 0);
            std::vector<jetgpu_group_task> tasks;
            std::vector<std::pair<size_t, uint64_t>> group_at(items.size()); // (first task, tiles)
            if (n_tasks) {
                const auto *tdev = static_cast<const int64_t *>(r.groups.get());
                for (size_t it = 0; it < items.size(); ++it) {
                    if (items[it].size() < 2)
                        continue;
                    group_at[it] = {tasks.size(), 0};
                    for (size_t i : items[it]) {
                        const auto &step = r.steps[i];
                        const auto &l = step.layout;
                        jetgpu_group_task q;
                        q.A = ptr(step.a);
                        q.B = ptr(step.b);
                        q.C = ptr(step.out);
                        q.batch = 1;
                        q.m = l.m;
                        q.n = l.n;
                        q.k = l.k;
                        q.a_bat = tdev;
                        q.a_row = tdev + table_at[i][0];
                        q.a_col = tdev + table_at[i][1];
                        q.b_bat = tdev;
                        q.b_row = tdev + table_at[i][2];
                        q.b_col = tdev + table_at[i][3];
                        tasks.push_back(q);
                        group_at[it].second += jetgpu_group_tiles(1, l.m, l.n);
                    }
                }
                Gpu::Check(jetgpu_memcpy(r.groups.get(), tables.data(),
                                         tables.size() * sizeof(int64_t), 0, Gpu::Stream()),
                           "group tables");
                Gpu::Check(jetgpu_memcpy(static_cast<char *>(r.groups.get()) + tables_bytes,
                                         tasks.data(), tasks.size() * sizeof(jetgpu_group_task),
                                         0, Gpu::Stream()),
                           "group tasks");
            }
            Gpu::Synchronize();
            const auto *task_dev = reinterpret_cast<const jetgpu_group_task *>(
                static_cast<const char *>(r.groups.get()) + tables_bytes);
            void *st = Gpu::Stream();
            Gpu::Check(jetgpu_graph_begin(st), "capture begin");
            for (size_t it = 0; it < items.size(); ++it) {
                const auto &item = items[it];
                if (item.size() >= 2) {
                    Gpu::Check(jetgpu_contract_group(task_dev + group_at[it].first,
                                                     (int)item.size(), group_at[it].second, dt,
                                                     st),
                               "grouped tiny steps (capture)");
                }
                else {
                    const auto &step = r.steps[item[0]];
                    const auto &l = step.layout;
                    Gpu::Check(jetgpu_contract(ptr(step.a), (int)l.a_shape.size(),
                                               l.a_shape.data(), l.a_perm.data(), ptr(step.b),
                                               (int)l.b_shape.size(), l.b_shape.data(),
                                               l.b_perm.data(), ptr(step.out), l.m, l.n, l.k, dt,
                                               r.precision, JETGPU_ALGO_4M, 0, 0, r.ws.get(),
                                               r.ws.size(), st),
                               "ContractTensors (capture)");
                }
                for (size_t i : item)
                    for (size_t q = 0; q < r.stores.size(); ++q)
                        if (r.stores[q].first == r.steps[i].out)
                            Gpu::Check(jetgpu_memcpy(result_ptr[q], ptr(r.steps[i].out),
                                                     r.bytes[r.steps[i].out], 2, st),
                                       "result copy (capture)");
            }
            Gpu::Check(jetgpu_graph_end(st, &r.graph), "capture end");
        }
    }
    size_t num_threads_;
    std::vector<Task> tasks_;
    NameToTaskMap name_to_task_;
    NameToTensorMap name_to_tensor_;
    NameToParentsMap name_to_parents_;
    std::vector<TensorType> results_;
    TensorType reduction_result_;
    double flops_ = 0;
    double memory_ = 0;
    bool reduced_ = false;

    static std::string TaskName(const PathStepInfo &s) { return std::to_string(s.id) + ":" + s.name; }

    void Run()
    {
        Gpu::Range range("Jet::TaskBasedContractor::Contract");
        // Index of the last contraction task consuming each name: its
        // deletion may run right after that task is enqueued.
        std::unordered_map<std::string, size_t> last_use;
        std::vector<const Task *> deletions;
        for (size_t t = 0; t < tasks_.size(); ++t) {
            const Task &task = tasks_[t];
            if (task.kind == Task::CONTRACT) {
                last_use[task.input_1] = t;
                last_use[task.input_2] = t;
            }
            else if (task.kind == Task::DELETE) {
                deletions.push_back(&task);
            }
        }
        std::unordered_map<size_t, std::vector<std::string>> delete_after;
        for (const Task *d : deletions) {
            const auto it = last_use.find(d->input_1);
            if (it != last_use.end())
                delete_after[it->second].push_back(d->input_1);
        }
        for (size_t t = 0; t < tasks_.size(); ++t) {
            const Task &task = tasks_[t];
            if (task.kind == Task::CONTRACT) {
                const TensorType &a = *name_to_tensor_.at(task.input_1);
                const TensorType &b = *name_to_tensor_.at(task.input_2);
                name_to_tensor_[task.name] =
                    std::make_unique<TensorType>(TensorType::ContractTensors(a, b));
                const auto it = delete_after.find(t);
                if (it != delete_after.end())
                    for (const auto &name : it->second) {
                        if constexpr (kGpuTensor) {
                            const auto slot = replay_.leaf_slot.find(name);
                            if (keep_leaves_ && slot != replay_.leaf_slot.end()) {
                                replay_.owned[slot->second] = std::move(name_to_tensor_[name]);
                                continue;
                            }
                        }
                        name_to_tensor_[name] = nullptr;
                    }
            }
            else if (task.kind == Task::STORE) {
                results_[task.result_id] = *name_to_tensor_.at(task.name);
            }
        }
        for (const Task &task : tasks_)
            if (task.kind == Task::REDUCE)
                Reduce();
        if constexpr (std::is_same_v<TensorType, Tensor<typename TensorType::scalar_type_t>>)
            Gpu::Synchronize();
    }

    void Reduce()
    {
        if (results_.empty())
            return;
        using T = typename TensorType::scalar_type_t;
        bool uniform = true;
        for (const auto &r : results_)
            uniform = uniform && r.GetIndices() == results_[0].GetIndices() &&
                      r.GetShape() == results_[0].GetShape();
        if constexpr (std::is_same_v<TensorType, Tensor<T>>) {
            const size_t size = results_[0].GetSize();
            if (uniform && size <= (size_t(1) << 22)) {
                // FP64 accumulation on the device, one pass per result.
                Gpu::DeviceBuffer acc(size * 16);
                for (size_t i = 0; i < results_.size(); ++i)
                    Gpu::Check(jetgpu_slice_sum_f64(results_[i].GetDeviceData(), 1, size,
                                                    Gpu::DtypeCode<T>(), acc.get(), i > 0 ? 1 : 0,
                                                    Gpu::Stream()),
                               "reduction");
                std::vector<std::complex<double>> host(size);
                Gpu::Check(jetgpu_memcpy(host.data(), acc.get(), size * 16, 1, Gpu::Stream()),
                           "reduction download");
                Gpu::Synchronize();
                std::vector<T> data(size);
                for (size_t i = 0; i < size; ++i)
                    data[i] = T(host[i]);
                reduction_result_ = TensorType(results_[0].GetIndices(), results_[0].GetShape(), data);
                return;
            }
        }
        TensorType acc;
        for (const auto &r : results_)
            acc = acc.AddTensor(r);
        reduction_result_ = std::move(acc);
    }
};

// The task dependency graph in DOT format (reference TaskBasedContractor.hpp:429-452,
// which prints Taskflow's dump). One node per task, labelled with its name;
// edges run from the task producing an operand to the task consuming it,
// from every result store to the reduction, and from every consumer of a
// tensor to that tensor's deletion task.
template <class TensorType>
inline std::ostream &operator<<(std::ostream &out, const TaskBasedContractor<TensorType> &tbc)
{
    using Task = typename TaskBasedContractor<TensorType>::Task;
    const auto &tasks = tbc.GetTasks();
    const auto &producer = tbc.GetNameToTaskMap();
    auto quoted = [](const std::string &s) {
        std::string q = "\"";
        for (char c : s) {
            if (c == '"' || c == '\\')
                q += '\\';
            q += c;
        }
        return q + "\"";
    };
    out << "digraph Taskflow {\n";
    for (size_t i = 0; i < tasks.size(); ++i) {
        std::string label = tasks[i].name;
        if (tasks[i].kind == Task::STORE)
            label = "store " + label;
        out << "t" << i << " [label=" << quoted(label) << "];\n";
    }
    for (size_t i = 0; i < tasks.size(); ++i) {
        const Task &t = tasks[i];
        if (t.kind == Task::CONTRACT) {
            for (const auto *in : {&t.input_1, &t.input_2}) {
                auto it = producer.find(*in);
                if (it != producer.end())
                    out << "t" << it->second << " -> t" << i << ";\n";
            }
        }
        else if (t.kind == Task::STORE) {
            out << "t" << producer.at(t.name) << " -> t" << i << ";\n";
        }
        else if (t.kind == Task::REDUCE) {
            for (size_t j = 0; j < tasks.size(); ++j)
                if (tasks[j].kind == Task::STORE)
                    out << "t" << j << " -> t" << i << ";\n";
        }
        else if (t.kind == Task::DELETE) {
            auto parents = tbc.GetNameToParentsMap().find(t.input_1);
            if (parents == tbc.GetNameToParentsMap().end())
                continue;
            for (const auto &consumer : parents->second) {
                auto it = producer.find(consumer);
                if (it != producer.end())
                    out << "t" << it->second << " -> t" << i << ";\n";
            }
        }
    }
    out << "}\n";
    return out;
}

} // namespace Jet
