// Jet::TensorNetwork (reference: include/jet/TensorNetwork.hpp): nodes, edges,
// tags, slicing and contraction along a path. Generic over the tensor type
// like the reference; with the device Jet::Tensor every slice and pairwise
// contraction runs on the GPU.
#pragma once

#include <string>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "Abort.hpp"
#include "Utilities.hpp"

namespace Jet {

template <class Tensor> class TensorNetwork {
  public:
    using NodeID_t = size_t;

    struct Node {
        NodeID_t id;
        std::string name;
        std::vector<std::string> indices;
        std::vector<std::string> tags;
        bool contracted;
        Tensor tensor;
    };

    struct Edge {
        size_t dim;
        std::vector<NodeID_t> node_ids;
        bool operator==(const Edge &o) const noexcept
        {
            std::unordered_set<size_t> a(node_ids.begin(), node_ids.end());
            std::unordered_set<size_t> b(o.node_ids.begin(), o.node_ids.end());
            return dim == o.dim && a == b;
        }
    };

    using Nodes = std::vector<Node>;
    using IndexToEdgeMap = std::unordered_map<std::string, Edge>;
    using TagToNodeIdsMap = std::unordered_multimap<std::string, NodeID_t>;
    using Path = std::vector<std::pair<NodeID_t, NodeID_t>>;

    const Nodes &GetNodes() const noexcept { return nodes_; }
    const IndexToEdgeMap &GetIndexToEdgeMap() const noexcept { return edges_; }
    const TagToNodeIdsMap &GetTagToNodesMap() const noexcept { return tags_; }
    const Path &GetPath() noexcept { return path_; }
    size_t NumIndices() const noexcept { return edges_.size(); }
    size_t NumTensors() const noexcept { return nodes_.size(); }

    NodeID_t AddTensor(const Tensor &tensor, const std::vector<std::string> &tags) noexcept
    {
        const NodeID_t id = nodes_.size();
        nodes_.push_back(Node{id, NameOf(tensor.GetIndices()), tensor.GetIndices(), tags, false,
                              tensor});
        RegisterEdges(nodes_.back());
        for (const auto &t : tags)
            tags_.emplace(t, id);
        return id;
    }

    // Fixes `indices` to the row-major unravel of `value` over their
    // dimensions (reference TensorNetwork.hpp:210-284): every node carrying a
    // sliced index keeps the sub-tensor (a device gather), its node labels
    // gain the "(value)" suffix and the sliced edges disappear.
    void SliceIndices(const std::vector<std::string> &indices, unsigned long long value)
    {
        std::vector<size_t> dims(indices.size());
        std::unordered_map<size_t, std::vector<size_t>> per_node;
        for (size_t i = 0; i < indices.size(); ++i) {
            const auto it = edges_.find(indices[i]);
            JET_ABORT_IF(it == edges_.end(), "Sliced index does not exist.");
            dims[i] = it->second.dim;
            for (NodeID_t id : it->second.node_ids)
                per_node[id].push_back(i);
        }
        const auto values = Utilities::UnravelIndex(value, dims);
        for (auto &[id, which] : per_node) {
            Node &node = nodes_[id];
            for (size_t i : which) {
                const std::string &label = indices[i];
                node.tensor = Tensor::SliceIndex(node.tensor, label, values[i]);
                for (auto &x : node.indices)
                    if (x == label)
                        x += "(" + std::to_string(values[i]) + ")";
            }
            node.name = NameOf(node.indices);
        }
        for (const auto &x : indices)
            edges_.erase(x);
    }

    // Contracts along `path` (pairs of node ids; each contraction appends a
    // node) or, with an empty path, every shared edge and then the scalars
    // (reference TensorNetwork.hpp:301-328, 461-518). Returns the last node.
    const Tensor &Contract(const Path &path = {})
    {
        JET_ABORT_IF(nodes_.empty(), "An empty tensor network cannot be contracted.");
        if (!path.empty()) {
            for (const auto &[a, b] : path) {
                JET_ABORT_IF_NOT(a < nodes_.size(), "Node ID 1 in contraction pair is invalid.");
                JET_ABORT_IF_NOT(b < nodes_.size(), "Node ID 2 in contraction pair is invalid.");
                const NodeID_t c = ContractPair(a, b);
                RewireAfter(a, b, c);
            }
            path_ = path;
        }
        else {
            std::vector<std::string> labels;
            for (const auto &kv : edges_)
                labels.push_back(kv.first);
            for (const auto &x : labels) {
                const auto it = edges_.find(x);
                if (it == edges_.end() || it->second.node_ids.size() != 2)
                    continue;
                const NodeID_t a = it->second.node_ids[0];
                const NodeID_t b = it->second.node_ids[1];
                const NodeID_t c = ContractPair(a, b);
                RewireAfter(a, b, c);
                path_.emplace_back(a, b);
            }
            std::vector<NodeID_t> scalars;
            for (const auto &n : nodes_)
                if (n.tensor.GetIndices().empty())
                    scalars.push_back(n.id);
            if (scalars.size() >= 2) {
                NodeID_t acc = scalars[0];
                for (size_t i = 1; i < scalars.size(); ++i) {
                    path_.emplace_back(acc, scalars[i]);
                    acc = ContractPair(acc, scalars[i]);
                }
            }
        }
        return nodes_.back().tensor;
    }

  private:
    Nodes nodes_;
    IndexToEdgeMap edges_;
    TagToNodeIdsMap tags_;
    Path path_;

    static std::string NameOf(const std::vector<std::string> &indices)
    {
        return indices.empty() ? std::string("_") : Utilities::JoinStringVector(indices);
    }

    void RegisterEdges(const Node &node)
    {
        const auto &shape = node.tensor.GetShape();
        for (size_t i = 0; i < node.indices.size(); ++i) {
            if (shape[i] < 2)
                continue; // dimension-1 indices form no edge
            auto it = edges_.find(node.indices[i]);
            if (it == edges_.end())
                edges_.emplace(node.indices[i], Edge{shape[i], {node.id}});
            else
                it->second.node_ids.push_back(node.id);
        }
    }

    NodeID_t ContractPair(NodeID_t a, NodeID_t b)
    {
        Tensor t = Tensor::ContractTensors(nodes_[a].tensor, nodes_[b].tensor);
        nodes_[a].contracted = true;
        nodes_[b].contracted = true;
        const auto idx = Utilities::VectorDisjunctiveUnion(nodes_[a].indices, nodes_[b].indices);
        const auto tags = Utilities::VectorUnion(nodes_[a].tags, nodes_[b].tags);
        const NodeID_t id = nodes_.size();
        nodes_.push_back(Node{id, NameOf(idx), idx, tags, false, std::move(t)});
        return id;
    }

    void RewireAfter(NodeID_t a, NodeID_t b, NodeID_t c)
    {
        for (const auto &x : nodes_[c].indices) {
            auto it = edges_.find(x);
            if (it == edges_.end())
                continue;
            for (auto &id : it->second.node_ids)
                if (id == a || id == b)
                    id = c;
        }
        for (const auto &x : Utilities::VectorIntersection(nodes_[a].tensor.GetIndices(),
                                                           nodes_[b].tensor.GetIndices()))
            edges_.erase(x);
    }
};

} // namespace Jet
