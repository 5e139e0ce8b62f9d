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
#pragma once

#include <future>
#include <memory>
#include <ostream>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "PathInfo.hpp"
#include "Tensor.hpp"
#include "TensorNetwork.hpp"

namespace Jet {

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
        const auto &nodes = tn.GetNodes();
        const size_t num_leaves = nodes.size();
        const size_t result_id = results_.size();
        results_.resize(result_id + 1);
        size_t shared = 0;
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
                name_to_tensor_.try_emplace(name_1,
                                            std::make_unique<TensorType>(nodes[id_1].tensor));
            if (id_2 < num_leaves)
                name_to_tensor_.try_emplace(name_2,
                                            std::make_unique<TensorType>(nodes[id_2].tensor));
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
        return shared;
    }

    size_t AddReductionTask() noexcept
    {
        if (reduced_)
            return 0;
        reduced_ = true;
        tasks_.push_back(Task{Task::REDUCE, "reduce", "", "", 0});
        return 1;
    }

    size_t AddDeletionTasks() noexcept
    {
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
        return std::async(std::launch::async, [this] { Run(); });
    }

  private:
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
                    for (const auto &name : it->second)
                        name_to_tensor_[name] = nullptr;
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
