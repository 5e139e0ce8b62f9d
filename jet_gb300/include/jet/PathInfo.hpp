// Jet::PathInfo (reference: include/jet/PathInfo.hpp): the step tree of a
// contraction path with per-step labels, flop and memory estimates. It also
// sizes the device memory of the contraction executors.
#pragma once

#include <limits>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "Abort.hpp"
#include "TensorNetwork.hpp"
#include "Utilities.hpp"

namespace Jet {

struct PathStepInfo {
    size_t id;
    size_t parent;
    std::pair<size_t, size_t> children;
    std::string name;
    std::vector<std::string> node_indices;
    std::vector<std::string> tensor_indices;
    std::vector<std::string> tags;
    std::vector<std::string> contracted_indices;
    static constexpr size_t MISSING_ID = std::numeric_limits<size_t>::max();
};

class PathInfo {
  public:
    using NodeID_t = size_t;
    using Path = std::vector<std::pair<NodeID_t, NodeID_t>>;
    using IndexToSizeMap = std::unordered_map<std::string, size_t>;
    using Steps = std::vector<PathStepInfo>;

    PathInfo() = default;

    template <class Tensor> PathInfo(const TensorNetwork<Tensor> &tn, const Path &path) : path_(path)
    {
        const auto &nodes = tn.GetNodes();
        num_leaves_ = nodes.size();
        steps_.reserve(num_leaves_ + path.size());
        for (const auto &n : nodes)
            steps_.push_back(PathStepInfo{n.id, PathStepInfo::MISSING_ID,
                                          {PathStepInfo::MISSING_ID, PathStepInfo::MISSING_ID},
                                          n.name, n.indices, n.tensor.GetIndices(), n.tags, {}});
        for (const auto &kv : tn.GetIndexToEdgeMap())
            sizes_.emplace(kv.first, kv.second.dim);
        for (const auto &[a, b] : path) {
            JET_ABORT_IF_NOT(a < steps_.size(), "Node ID 1 in contraction path pair is invalid.");
            JET_ABORT_IF_NOT(b < steps_.size(), "Node ID 2 in contraction path pair is invalid.");
            Merge(a, b);
        }
    }

    const IndexToSizeMap &GetIndexSizes() const noexcept { return sizes_; }
    size_t GetNumLeaves() const noexcept { return num_leaves_; }
    const Path &GetPath() const noexcept { return path_; }
    const Steps &GetSteps() const noexcept { return steps_; }

    // size(out) * 2 * prod(contracted dims): complex multiply-adds counted as 2.
    double GetPathStepFlops(size_t id) const
    {
        JET_ABORT_IF_NOT(id < steps_.size(), "Step ID is invalid.");
        if (id < num_leaves_)
            return 0;
        const double muls = Product(steps_[id].contracted_indices);
        return Product(steps_[id].tensor_indices) * (muls + muls);
    }

    double GetTotalFlops() const noexcept
    {
        double f = 0;
        for (size_t i = num_leaves_; i < steps_.size(); ++i)
            f += GetPathStepFlops(i);
        return f;
    }

    double GetPathStepMemory(size_t id) const
    {
        JET_ABORT_IF_NOT(id < steps_.size(), "Step ID is invalid.");
        return Product(steps_[id].tensor_indices);
    }

    double GetTotalMemory() const noexcept
    {
        double m = 0;
        for (size_t i = 0; i < steps_.size(); ++i)
            m += GetPathStepMemory(i);
        return m;
    }

  private:
    Path path_;
    Steps steps_;
    size_t num_leaves_ = 0;
    IndexToSizeMap sizes_;

    double Product(const std::vector<std::string> &labels) const
    {
        double p = 1;
        for (const auto &x : labels) {
            const auto it = sizes_.find(x);
            p *= it == sizes_.end() ? 1.0 : (double)it->second;
        }
        return p;
    }

    void Merge(size_t a, size_t b)
    {
        using namespace Utilities;
        const size_t id = steps_.size();
        auto &s1 = steps_[a];
        auto &s2 = steps_[b];
        const auto contracted = VectorIntersection(s1.tensor_indices, s2.tensor_indices);
        const auto node_idx =
            VectorSubtraction(VectorConcatenation(s1.node_indices, s2.node_indices), contracted);
        const auto tensor_idx = VectorDisjunctiveUnion(s1.tensor_indices, s2.tensor_indices);
        const auto tags = VectorUnion(s1.tags, s2.tags);
        s1.parent = id;
        s2.parent = id;
        steps_.push_back(PathStepInfo{id, PathStepInfo::MISSING_ID, {a, b},
                                      node_idx.empty() ? std::string("_")
                                                       : JoinStringVector(node_idx),
                                      node_idx, tensor_idx, tags, contracted});
    }
};

} // namespace Jet
