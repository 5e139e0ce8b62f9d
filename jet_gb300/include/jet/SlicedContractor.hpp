// Jet::SlicedContractor: all slices of a sliced network along one path, as
// batched GPU launches replayed from one captured CUDA graph.
//
// The reference contracts a sliced network by building one TensorNetwork per
// slice value (TensorNetwork::SliceIndices, TensorNetwork.hpp:210-284), adding
// every copy to a TaskBasedContractor -- which shares the tasks whose names
// coincide, i.e. the slice-independent subtrees (TaskBasedContractor.hpp:
// 218-222) -- and summing the results with AddTensors (:258-280).
//
// Here the slice value becomes a label of its own, "$s", carried by every
// leaf that touches a sliced index (its sliced axes are gathered on the device
// for a chunk of B consecutive slice values: jetgpu_slice_gather_at) and by
// every intermediate that depends on such a leaf. "$s" is never contracted:
//   * on one operand only, it is an ordinary free index and folds into the
//     rows or columns of the product (slice-independent operands are shared
//     by the whole chunk, computed once -- the reference's task sharing);
//   * on both operands, it is the batch dimension of jetgpu_contract_batched.
// Leaves may also carry alternatives ("$b", e.g. the output caps of several
// bitstrings): "$b" behaves the same way and stays in the result, so one run
// yields one amplitude per alternative while sharing every
// alternative-independent intermediate.
//
// Execution: steps whose output has no "$s" run once (stream-ordered). The
// "$s" steps run per chunk from one CUDA graph captured over fixed buffers (a
// liveness-planned arena sized from the step sizes of the path, i.e. PathInfo's
// memory per step times B); the graph ends with the FP64 sum over the chunk's
// slices into the accumulator and advances the device slice counter, so the
// host just replays it chunk after chunk.
#pragma once

#include <algorithm>
#include <array>
#include <complex>
#include <limits>
#include <map>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "GroupSchedule.hpp"
#include "PathInfo.hpp"
#include "Tensor.hpp"
#include "TensorNetwork.hpp"

namespace Jet {

template <class T = std::complex<float>> class SlicedContractor {
  public:
    static constexpr const char *kSlice = "$s";
    static constexpr const char *kAlt = "$b";

    SlicedContractor(const TensorNetwork<Tensor<T>> &tn, const PathInfo::Path &path,
                     const std::vector<std::string> &sliced, int precision = JETGPU_PREC_FP32)
        : path_(path), sliced_(sliced), precision_(precision)
    {
        JET_ABORT_IF(path.empty(), "SlicedContractor needs a contraction path.");
        const auto &nodes = tn.GetNodes();
        num_leaves_ = nodes.size();
        const auto &edges = tn.GetIndexToEdgeMap();
        slice_dims_.resize(sliced.size());
        num_slices_ = 1;
        for (size_t i = 0; i < sliced.size(); ++i) {
            const auto it = edges.find(sliced[i]);
            JET_ABORT_IF(it == edges.end(), "Sliced index does not exist.");
            slice_dims_[i] = it->second.dim;
            num_slices_ *= slice_dims_[i];
        }
        slice_strides_.assign(sliced.size(), 1);
        for (size_t i = sliced.size(); i-- > 1;)
            slice_strides_[i - 1] = slice_strides_[i] * slice_dims_[i];
        for (const auto &n : nodes)
            leaves_.push_back(n.tensor);
        alt_values_.resize(num_leaves_);
        batch_ = std::min<size_t>(num_slices_, 64);
    }

    ~SlicedContractor() { ReleaseGraph(); }
    SlicedContractor(const SlicedContractor &) = delete;
    SlicedContractor &operator=(const SlicedContractor &) = delete;

    // Leaf `node_id` takes `n_alt` alternative values (n_alt x leaf size,
    // row-major); the result gains a "$b" axis of n_alt.
    void SetLeafAlternatives(size_t node_id, const std::vector<T> &values, size_t n_alt)
    {
        JET_ABORT_IF_NOT(node_id < num_leaves_, "Node ID is invalid.");
        JET_ABORT_IF_NOT(values.size() == n_alt * leaves_[node_id].GetSize(),
                         "Alternative values do not match the leaf size.");
        JET_ABORT_IF(n_alt_ != 0 && n_alt_ != n_alt,
                     "All leaves with alternatives must have the same count.");
        for (const auto &x : leaves_[node_id].GetIndices())
            JET_ABORT_IF(std::find(sliced_.begin(), sliced_.end(), x) != sliced_.end(),
                         "A leaf with alternatives cannot carry a sliced index.");
        n_alt_ = n_alt;
        alt_values_[node_id] = values;
        planned_ = false;
    }

    // Slices per batched launch (a divisor of the slice count is used).
    void SetBatchSize(size_t b)
    {
        batch_ = std::max<size_t>(1, std::min(b, num_slices_));
        while (num_slices_ % batch_)
            --batch_;
        planned_ = false;
    }

    size_t GetBatchSize() const { return batch_; }

    // Run consecutive independent tiny steps (AUTO / TUNED / FP32 only) as
    // one grouped launch (default on; off: one launch per step).
    void SetGrouping(bool on)
    {
        grouping_ = on;
        planned_ = false;
    }

    // Pass each step's recorded output exponent to the steps consuming it, so
    // the FP16x3 form skips its scan of tensor-core outputs (default on; the
    // results are the same either way).
    void SetExponentHints(bool on)
    {
        exponent_hints_ = on;
        ReleaseGraph();
    }
    size_t GetNumSlices() const { return num_slices_; }

    // Sum over slices [first, first + count) of the network's result, in FP64.
    // count must be a multiple of the batch size.
    std::vector<std::complex<double>> Contract(size_t first = 0, size_t count = SIZE_MAX)
    {
        if (count == SIZE_MAX)
            count = num_slices_ - first;
        JET_ABORT_IF(first + count > num_slices_, "Slice range out of bounds.");
        JET_ABORT_IF(count % batch_ != 0, "Slice count must be a multiple of the batch size.");
        Gpu::Range range("Jet::SlicedContractor::Contract");
        if (!planned_)
            Plan();
        void *st = Gpu::Stream();
        RunPrefix(st);
        Gpu::Check(jetgpu_memset_zero(acc_.get(), result_size_ * 16, st), "zero accumulator");
        if (sliced_.empty()) {
            // No slicing: the whole path ran as prefix steps.
            Gpu::Check(jetgpu_slice_sum_f64(Buffer(final_id_), 1, result_size_,
                                            Gpu::DtypeCode<T>(), acc_.get(), 0, st),
                       "result");
        }
        else {
            const uint64_t first64 = first;
            Gpu::Check(jetgpu_memcpy(counter_.get(), &first64, 8, 0, st), "slice counter");
            if (graph_ == nullptr)
                Capture(st);
            for (size_t c = 0; c < count / batch_; ++c)
                Gpu::Check(jetgpu_graph_launch(graph_, st), "graph launch");
        }
        std::vector<std::complex<double>> out(result_size_);
        Gpu::Check(jetgpu_memcpy(out.data(), acc_.get(), result_size_ * 16, 1, st), "download");
        Gpu::Synchronize();
        return out;
    }

    // One entry of ProfileChunk: a slice gather ("gather"), a path step
    // ("contract"), a grouped launch of tiny steps ("group": `step` is its
    // first step, `batch` the number of steps), the result reorder ("result
    // reorder") or the FP64 slice sum ("slice sum").
    struct ChunkProfileEntry {
        std::string kind;
        int step; // index into the path (-1 when not a step)
        uint64_t batch, m, n, k;
        double ms;
    };

    // Runs one chunk (slices [first, first + batch size)) eagerly with a CUDA
    // event after every gather, contraction and the slice sum, and
    // returns each one's device time: a per-step profile of what the captured
    // graph replays. The accumulator holds that chunk's sum afterwards.
    std::vector<ChunkProfileEntry> ProfileChunk(size_t first = 0)
    {
        JET_ABORT_IF(first % batch_ != 0 || first + batch_ > num_slices_,
                     "Chunk start must be a multiple of the batch size inside the slice range.");
        JET_ABORT_IF(sliced_.empty(), "A network without sliced indices has no chunk.");
        Gpu::Range range("Jet::SlicedContractor::ProfileChunk");
        if (!planned_)
            Plan();
        void *st = Gpu::Stream();
        RunPrefix(st);
        Gpu::Check(jetgpu_memset_zero(acc_.get(), result_size_ * 16, st), "zero accumulator");
        const uint64_t first64 = first;
        Gpu::Check(jetgpu_memcpy(counter_.get(), &first64, 8, 0, st), "slice counter");
        Profile prof(st);
        RecordChunk(st, &prof);
        const std::vector<double> ms = prof.timer.Finish();
        for (size_t i = 0; i < prof.entries.size(); ++i)
            prof.entries[i].ms = ms[i];
        return prof.entries;
    }

    // Labels and shape of the result (the "$b" axis, if any, included).
    const std::vector<std::string> &GetResultIndices() const { return result_labels_; }
    const std::vector<size_t> &GetResultShape() const { return result_dims_; }

    // Flops of one slice, PathInfo's convention (size(out) * 2 * prod(contracted)).
    double GetSliceFlops()
    {
        if (!planned_)
            Plan();
        return slice_flops_;
    }
    // Flops of the steps that depend on the slice (repeated per slice).
    double GetSliceDependentFlops()
    {
        if (!planned_)
            Plan();
        return slice_dep_flops_;
    }
    size_t GetArenaBytes()
    {
        if (!planned_)
            Plan();
        return arena_bytes_;
    }

    // Device bytes a contraction at the current batch size holds: the chunk
    // arena, the largest step's workspace, the slice-independent buffers and
    // the prefix's peak of transient intermediates. Planned without
    // allocating, so slice counts and batch sizes can be chosen against a
    // memory budget before any of it is committed.
    size_t EstimateDeviceBytes()
    {
        if (!planned_)
            Plan(false);
        size_t persistent = 0, transient = 0, peak = 0;
        for (size_t i = 0; i < nodes_.size(); ++i)
            if (!nodes_[i].chunk && persist_[i])
                persistent += nodes_[i].bytes;
        for (size_t i = 0; i < steps_.size(); ++i) {
            const Step &st = steps_[i];
            if (st.chunk)
                continue;
            if (!persist_[st.out])
                transient += nodes_[st.out].bytes;
            peak = std::max(peak, transient);
            for (int id : {st.a, st.b})
                if (!persist_[id] && prefix_last_use_[id] == (int)i)
                    transient -= nodes_[id].bytes;
        }
        return arena_bytes_ + ws_bytes_ + persistent + peak + result_size_ * 16;
    }

  private:
    struct Node {
        std::vector<std::string> labels;
        std::vector<uint64_t> dims;
        bool chunk = false; // carries "$s"
        size_t bytes = 0;
        size_t offset = 0; // in the chunk arena
        Gpu::DeviceBuffer own; // prefix tensors and leaves
    };
    struct Step {
        int a, b, out;
        bool chunk;
        bool batched; // "$s"/"$b" on both operands
        uint64_t batch, m, n, k;
        // Operand views passed to the product, and how each carries the batch
        // (jetgpu_contract_batched's a_batched / b_batched: 0 shared, 1
        // tensors back to back, 2 batch axes leading the permutation).
        std::vector<uint64_t> a_shape, b_shape;
        std::vector<int32_t> a_perm, b_perm;
        int a_mode = 0, b_mode = 0;
        size_t ws = 0;
        // Labels of the product's view: batch (hyper), rows, k, columns.
        std::vector<std::string> hyper, left, common, right;
    };
    // What one chunk replays, in order: one step, or a group of independent
    // tiny steps run as one grouped launch (jetgpu_contract_group).
    struct Item {
        std::vector<int> steps;
        bool grouped = false;
        const jetgpu_group_task *tasks = nullptr; // device task table (grouped)
        uint64_t tiles = 0;
    };
    struct Profile {
        explicit Profile(void *st) : timer(st) {}
        Gpu::StreamTimer timer;
        std::vector<ChunkProfileEntry> entries;
        void Mark(const char *kind, int step, uint64_t b, uint64_t m, uint64_t n, uint64_t k)
        {
            timer.Mark();
            entries.push_back(ChunkProfileEntry{kind, step, b, m, n, k, 0.0});
        }
    };
    struct Loader { // a "$s" leaf gathered per chunk
        int leaf;
        std::vector<uint64_t> shape;
        std::vector<int32_t> axes;
        std::vector<uint64_t> value_strides;
    };

    PathInfo::Path path_;
    std::vector<std::string> sliced_;
    std::vector<uint64_t> slice_dims_, slice_strides_;
    size_t num_slices_ = 1, num_leaves_ = 0, batch_ = 1, n_alt_ = 0;
    int precision_;
    std::vector<Tensor<T>> leaves_;
    std::vector<std::vector<T>> alt_values_;
    std::vector<Node> nodes_;
    std::vector<Step> steps_;
    std::vector<Loader> loaders_;
    int final_id_ = -1;
    int final_perm_needed_ = 0;
    std::vector<uint64_t> final_shape_;
    std::vector<int32_t> final_perm_;
    std::vector<std::string> result_labels_;
    std::vector<size_t> result_dims_;
    size_t result_size_ = 1;
    double slice_flops_ = 0, slice_dep_flops_ = 0;
    size_t arena_bytes_ = 0, ws_bytes_ = 0;
    bool planned_ = false;
    bool prefix_done_ = false;
    std::vector<char> persist_;
    std::vector<int> prefix_last_use_;
    Gpu::DeviceBuffer arena_, ws_, acc_, counter_, final_tmp_;
    // One int per node: the max exponent its producing step recorded
    // (jetgpu_contract_batched_hinted), read by the steps consuming it.
    Gpu::DeviceBuffer emax_;
    bool exponent_hints_ = true;
    // Grouped launches of tiny steps (jetgpu_contract_group).
    static constexpr double kGroupMaxWork = 131072.0; // batch m n k below AUTO's smallest TC step
    std::vector<Item> items_;
    Gpu::DeviceBuffer group_buf_;
    bool grouping_ = true;
    std::vector<Gpu::DeviceBuffer> alt_bufs_;
    void *graph_ = nullptr;

    static bool IsHyper(const std::string &x) { return x == kSlice || x == kAlt; }

    uint64_t Dim(const Node &n, const std::string &x) const
    {
        for (size_t i = 0; i < n.labels.size(); ++i)
            if (n.labels[i] == x)
                return n.dims[i];
        return 1;
    }

    static int32_t Pos(const std::vector<std::string> &v, const std::string &x)
    {
        return static_cast<int32_t>(std::find(v.begin(), v.end(), x) - v.begin());
    }

    void *Buffer(int id)
    {
        Node &n = nodes_[id];
        if (n.chunk)
            return static_cast<char *>(arena_.get()) + n.offset;
        return n.own.get();
    }

    void ReleaseGraph()
    {
        if (graph_)
            jetgpu_graph_destroy(graph_);
        graph_ = nullptr;
    }

    // allocate = false computes the layout only (EstimateDeviceBytes); the
    // contractor then stays unplanned.
    void Plan(bool allocate = true)
    {
        using namespace Utilities;
        ReleaseGraph();
        nodes_.clear();
        steps_.clear();
        loaders_.clear();
        alt_bufs_.clear();
        const int dt = Gpu::DtypeCode<T>();
        const size_t eb = sizeof(T);
        // Leaves.
        nodes_.resize(num_leaves_);
        for (size_t i = 0; i < num_leaves_; ++i) {
            Node &n = nodes_[i];
            const auto &lab = leaves_[i].GetIndices();
            const auto &sh = leaves_[i].GetShape();
            Loader ld;
            ld.leaf = (int)i;
            std::vector<std::string> rest;
            std::vector<uint64_t> rest_dims;
            for (size_t a = 0; a < lab.size(); ++a) {
                const auto it = std::find(sliced_.begin(), sliced_.end(), lab[a]);
                if (it != sliced_.end()) {
                    ld.axes.push_back((int32_t)a);
                    ld.value_strides.push_back(slice_strides_[it - sliced_.begin()]);
                }
                else {
                    rest.push_back(lab[a]);
                    rest_dims.push_back(sh[a]);
                }
            }
            if (!ld.axes.empty()) {
                n.labels = {kSlice};
                n.dims = {batch_};
                n.chunk = true;
                ld.shape.assign(sh.begin(), sh.end());
                loaders_.push_back(ld);
            }
            else if (!alt_values_[i].empty()) {
                n.labels = {kAlt};
                n.dims = {n_alt_};
            }
            n.labels.insert(n.labels.end(), rest.begin(), rest.end());
            n.dims.insert(n.dims.end(), rest_dims.begin(), rest_dims.end());
            n.bytes = eb;
            for (auto d : n.dims)
                n.bytes *= d;
        }
        // Steps (symbolic).
        slice_flops_ = slice_dep_flops_ = 0;
        ws_bytes_ = 0;
        for (size_t i = 0; i < path_.size(); ++i) {
            const auto [ia, ib] = path_[i];
            JET_ABORT_IF_NOT(ia < nodes_.size() && ib < nodes_.size(),
                             "Node ID in contraction path pair is invalid.");
            // References stay valid: nodes_ grows only at the end of the body.
            const Node &A = nodes_[ia];
            const Node &B = nodes_[ib];
            Step s;
            s.a = (int)ia;
            s.b = (int)ib;
            s.out = (int)nodes_.size();
            const auto shared = VectorIntersection(A.labels, B.labels);
            std::vector<std::string> hyper, common;
            for (const auto &x : shared)
                (IsHyper(x) ? hyper : common).push_back(x);
            const auto left = VectorSubtraction(A.labels, B.labels);
            const auto right = VectorSubtraction(B.labels, A.labels);
            Node out;
            s.batched = !hyper.empty();
            s.batch = 1;
            for (const auto &x : hyper)
                s.batch *= Dim(A, x);
            s.m = s.n = s.k = 1;
            for (const auto &x : left)
                s.m *= Dim(A, x);
            for (const auto &x : right)
                s.n *= Dim(B, x);
            for (const auto &x : common)
                s.k *= Dim(A, x);
            out.labels = VectorConcatenation(hyper, VectorConcatenation(left, right));
            for (const auto &x : hyper)
                out.dims.push_back(Dim(A, x));
            for (const auto &x : left)
                out.dims.push_back(Dim(A, x));
            for (const auto &x : right)
                out.dims.push_back(Dim(B, x));
            // Operand views.
            auto view = [&](const Node &X, const std::vector<std::string> &order,
                            std::vector<uint64_t> &shape, std::vector<int32_t> &perm) {
                // The product wants X as `hyper` (the batch) followed by `order`.
                // With hyper leading X's labels, X is batch tensors back to back
                // (mode 1); otherwise the batch axes lead X's permutation and
                // the product's own permute pass moves them (mode 2).
                const bool leading = X.labels.size() >= hyper.size() &&
                                     std::equal(hyper.begin(), hyper.end(), X.labels.begin());
                if (leading) {
                    const std::vector<std::string> body(X.labels.begin() + hyper.size(),
                                                        X.labels.end());
                    for (const auto &x : body)
                        shape.push_back(Dim(X, x));
                    for (const auto &x : order)
                        perm.push_back(Pos(body, x));
                    return 1;
                }
                shape = X.dims;
                for (const auto &x : hyper)
                    perm.push_back(Pos(X.labels, x));
                for (const auto &x : order)
                    perm.push_back(Pos(X.labels, x));
                return 2;
            };
            s.a_mode = view(A, VectorConcatenation(left, common), s.a_shape, s.a_perm);
            s.b_mode = view(B, VectorConcatenation(common, right), s.b_shape, s.b_perm);
            if (!s.batched)
                s.a_mode = s.b_mode = 0;
            s.hyper = hyper;
            s.left = left;
            s.common = common;
            s.right = right;
            s.ws = jetgpu_contract_batched_workspace_size(
                s.batch, (int)s.a_shape.size(), s.a_shape.data(), s.a_perm.data(), s.a_mode,
                (int)s.b_shape.size(), s.b_shape.data(), s.b_perm.data(), s.b_mode, s.m, s.n,
                s.k, dt, precision_);
            ws_bytes_ = std::max(ws_bytes_, s.ws);
            out.chunk = InVector(std::string(kSlice), out.labels);
            s.chunk = out.chunk;
            out.bytes = eb;
            for (auto d : out.dims)
                out.bytes *= d;
            // Flops per slice: "$s" counts once, "$b" as itself.
            double fl = 2.0 * (double)s.k;
            for (size_t j = 0; j < out.labels.size(); ++j)
                fl *= out.labels[j] == kSlice ? 1.0 : (double)out.dims[j];
            slice_flops_ += fl;
            if (s.chunk)
                slice_dep_flops_ += fl;
            nodes_.push_back(std::move(out));
            steps_.push_back(std::move(s));
        }
        final_id_ = (int)nodes_.size() - 1;
        const Node &fin = nodes_[final_id_];
        // Result: the final tensor without "$s"; "$s" moved to the front for the sum.
        result_labels_.clear();
        result_dims_.clear();
        result_size_ = 1;
        final_perm_.clear();
        final_shape_ = fin.dims;
        const int spos = Pos(fin.labels, kSlice);
        if (spos < (int)fin.labels.size())
            final_perm_.push_back(spos);
        for (size_t j = 0; j < fin.labels.size(); ++j) {
            if ((int)j == spos)
                continue;
            final_perm_.push_back((int32_t)j);
            result_labels_.push_back(fin.labels[j]);
            result_dims_.push_back(fin.dims[j]);
            result_size_ *= fin.dims[j];
        }
        final_perm_needed_ = spos > 0 && spos < (int)fin.labels.size();
        // What a chunk replays: the tiny steps of a run, level by level, in
        // grouped launches (group_schedule::Items); every other step is its
        // own item. A level of one step keeps its own launch (split-k, tuned
        // forms).
        items_.clear();
        {
            std::vector<int> chunk_steps;
            for (size_t i = 0; i < steps_.size(); ++i)
                if (steps_[i].chunk)
                    chunk_steps.push_back((int)i);
            std::vector<char> groupable(chunk_steps.size());
            std::vector<std::array<size_t, 2>> inputs(chunk_steps.size());
            std::vector<size_t> outputs(chunk_steps.size());
            for (size_t j = 0; j < chunk_steps.size(); ++j) {
                const Step &st = steps_[chunk_steps[j]];
                groupable[j] = Groupable(st);
                inputs[j] = {(size_t)st.a, (size_t)st.b};
                outputs[j] = (size_t)st.out;
            }
            for (const auto &item : group_schedule::Items(groupable, inputs, outputs, 256)) {
                std::vector<int> ids;
                for (size_t j : item)
                    ids.push_back(chunk_steps[j]);
                items_.push_back(Item{ids, ids.size() > 1});
            }
        }
        // Chunk arena: liveness-planned offsets (first fit, 256-byte aligned)
        // over the items: a group's outputs are all live while it runs.
        std::vector<int> last_use(nodes_.size(), -1);
        for (size_t it = 0; it < items_.size(); ++it)
            for (int i : items_[it].steps) {
                last_use[steps_[i].a] = (int)it;
                last_use[steps_[i].b] = (int)it;
            }
        last_use[final_id_] = (int)items_.size();
        std::map<size_t, size_t> free_blocks; // offset -> size
        size_t top = 0;
        auto align = [](size_t v) { return (v + 255) / 256 * 256; };
        auto alloc = [&](size_t bytes) {
            bytes = align(bytes);
            for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it)
                if (it->second >= bytes) {
                    const size_t off = it->first;
                    const size_t rem = it->second - bytes;
                    free_blocks.erase(it);
                    if (rem)
                        free_blocks[off + bytes] = rem;
                    return off;
                }
            const size_t off = top;
            top += bytes;
            return off;
        };
        auto release = [&](size_t off, size_t bytes) {
            bytes = align(bytes);
            auto it = free_blocks.emplace(off, bytes).first;
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
        for (size_t i = 0; i < num_leaves_; ++i)
            if (nodes_[i].chunk)
                nodes_[i].offset = alloc(nodes_[i].bytes);
        for (size_t it = 0; it < items_.size(); ++it) {
            for (int i : items_[it].steps)
                nodes_[steps_[i].out].offset = alloc(nodes_[steps_[i].out].bytes);
            for (int i : items_[it].steps)
                for (int id : {steps_[i].a, steps_[i].b})
                    if (nodes_[id].chunk && last_use[id] == (int)it && id != final_id_) {
                        release(nodes_[id].offset, nodes_[id].bytes);
                        last_use[id] = -2; // released once
                    }
        }
        arena_bytes_ = top;
        if (!allocate) {
            PlanPersistence();
            return;
        }
        arena_ = Gpu::DeviceBuffer(std::max<size_t>(arena_bytes_, 256));
        ws_ = Gpu::DeviceBuffer(ws_bytes_);
        acc_ = Gpu::DeviceBuffer(std::max<size_t>(result_size_ * 16, 16));
        counter_ = Gpu::DeviceBuffer(8);
        emax_ = Gpu::DeviceBuffer(std::max<size_t>(nodes_.size(), 1) * sizeof(int));
        {
            // Nothing recorded yet (any value below -1000).
            const std::vector<int> unknown(std::max<size_t>(nodes_.size(), 1),
                                           std::numeric_limits<int>::min());
            Gpu::Check(jetgpu_memcpy(emax_.get(), unknown.data(), unknown.size() * sizeof(int),
                                     0, Gpu::Stream()),
                       "exponent slots");
            Gpu::Synchronize();
        }
        final_tmp_ = Gpu::DeviceBuffer(final_perm_needed_ ? nodes_[final_id_].bytes : 0);
        PlanPersistence();
        for (size_t i = 0; i < nodes_.size(); ++i)
            if (!nodes_[i].chunk && persist_[i])
                nodes_[i].own = Gpu::DeviceBuffer(nodes_[i].bytes);
        BuildGroups();
        prefix_done_ = false;
        planned_ = true;
    }

    // Slice-independent tensors that the captured graph reads (leaves,
    // prefix outputs consumed by "$s" steps, the final result) keep one
    // buffer for the contractor's lifetime; other prefix intermediates live
    // only while the prefix runs.
    void PlanPersistence()
    {
        persist_.assign(nodes_.size(), 0);
        for (size_t i = 0; i < num_leaves_; ++i)
            persist_[i] = 1;
        for (const Step &s : steps_)
            if (s.chunk)
                for (int id : {s.a, s.b})
                    persist_[id] = 1;
        persist_[final_id_] = 1;
        prefix_last_use_.assign(nodes_.size(), -1);
        for (size_t i = 0; i < steps_.size(); ++i)
            if (!steps_[i].chunk) {
                prefix_last_use_[steps_[i].a] = (int)i;
                prefix_last_use_[steps_[i].b] = (int)i;
            }
    }

    // Tiny slice-dependent steps that AUTO and TUNED give to the plain
    // product anyway (and every tiny step in plain FP32): one grouped launch
    // per run of two or more independent ones. (The grouped kernel has no
    // split-k: a long-k step alone keeps its own launch.)
    bool Groupable(const Step &st) const
    {
        if (!grouping_ || !(precision_ == JETGPU_PREC_FP32 || precision_ == JETGPU_PREC_AUTO ||
                            precision_ == JETGPU_PREC_TUNED))
            return false;
        return (double)st.batch * (double)st.m * (double)st.n * (double)st.k < kGroupMaxWork;
    }

    // Element offsets, in node X, of every index combination of `labels`
    // (first label slowest): a product view's batch, row or column table.
    static std::vector<int64_t> Offsets(const Node &X, const std::vector<std::string> &labels)
    {
        std::vector<int64_t> strides(X.dims.size());
        int64_t st = 1;
        for (size_t j = X.dims.size(); j-- > 0;) {
            strides[j] = st;
            st *= (int64_t)X.dims[j];
        }
        std::vector<int64_t> out{0};
        for (const auto &l : labels) {
            const size_t p = (size_t)Pos(X.labels, l);
            std::vector<int64_t> next;
            next.reserve(out.size() * X.dims[p]);
            for (int64_t o : out)
                for (uint64_t d = 0; d < X.dims[p]; ++d)
                    next.push_back(o + (int64_t)d * strides[p]);
            out.swap(next);
        }
        return out;
    }

    // Device task tables of the grouped items (offset tables, then tasks).
    void BuildGroups()
    {
        std::vector<int64_t> tables;
        struct Pending {
            size_t item;
            std::vector<std::array<size_t, 6>> table_at; // per task: 6 table offsets
        };
        std::vector<Pending> pend;
        for (size_t it = 0; it < items_.size(); ++it) {
            if (!items_[it].grouped)
                continue;
            Pending p{it, {}};
            for (int i : items_[it].steps) {
                const Step &st = steps_[i];
                const Node &A = nodes_[st.a], &B = nodes_[st.b];
                const std::vector<std::vector<int64_t>> t6{
                    Offsets(A, st.hyper), Offsets(A, st.left),   Offsets(A, st.common),
                    Offsets(B, st.hyper), Offsets(B, st.common), Offsets(B, st.right)};
                std::array<size_t, 6> at{};
                for (int q = 0; q < 6; ++q) {
                    at[q] = tables.size();
                    tables.insert(tables.end(), t6[q].begin(), t6[q].end());
                }
                p.table_at.push_back(at);
            }
            pend.push_back(std::move(p));
        }
        size_t n_tasks = 0;
        for (const auto &p : pend)
            n_tasks += p.table_at.size();
        const size_t tables_bytes = (tables.size() * sizeof(int64_t) + 255) / 256 * 256;
        group_buf_ = Gpu::DeviceBuffer(tables_bytes + n_tasks * sizeof(jetgpu_group_task));
        if (n_tasks == 0)
            return;
        const auto *tdev = static_cast<const int64_t *>(group_buf_.get());
        auto *task_dev = reinterpret_cast<jetgpu_group_task *>(
            static_cast<char *>(group_buf_.get()) + tables_bytes);
        std::vector<jetgpu_group_task> tasks;
        for (const auto &p : pend) {
            Item &item = items_[p.item];
            item.tasks = task_dev + tasks.size();
            item.tiles = 0;
            for (size_t j = 0; j < item.steps.size(); ++j) {
                const Step &st = steps_[item.steps[j]];
                const auto &at = p.table_at[j];
                jetgpu_group_task q;
                q.A = Buffer(st.a);
                q.B = Buffer(st.b);
                q.C = Buffer(st.out);
                q.batch = st.batch;
                q.m = st.m;
                q.n = st.n;
                q.k = st.k;
                q.a_bat = tdev + at[0];
                q.a_row = tdev + at[1];
                q.a_col = tdev + at[2];
                q.b_bat = tdev + at[3];
                q.b_row = tdev + at[4];
                q.b_col = tdev + at[5];
                tasks.push_back(q);
                item.tiles += jetgpu_group_tiles(st.batch, st.m, st.n);
            }
        }
        void *st = Gpu::Stream();
        if (!tables.empty())
            Gpu::Check(jetgpu_memcpy(group_buf_.get(), tables.data(),
                                     tables.size() * sizeof(int64_t), 0, st),
                       "group tables");
        Gpu::Check(jetgpu_memcpy(task_dev, tasks.data(), tasks.size() * sizeof(jetgpu_group_task),
                                 0, st),
                   "group tasks");
        Gpu::Synchronize();
    }

    // Runs every step whose output has no "$s" (once per Contract call) and
    // prepares the leaves.
    void RunPrefix(void *st)
    {
        if (prefix_done_)
            return;
        for (size_t i = 0; i < num_leaves_; ++i) {
            Node &n = nodes_[i];
            if (n.chunk)
                continue;
            if (!alt_values_[i].empty())
                Gpu::Check(jetgpu_memcpy(n.own.get(), alt_values_[i].data(), n.bytes, 0, st),
                           "upload alternatives");
            else
                Gpu::Check(jetgpu_memcpy(n.own.get(), leaves_[i].GetDeviceData(), n.bytes, 2, st),
                           "leaf copy");
        }
        for (size_t i = 0; i < steps_.size(); ++i) {
            const Step &s = steps_[i];
            if (s.chunk)
                continue;
            if (!persist_[s.out])
                nodes_[s.out].own = Gpu::DeviceBuffer(nodes_[s.out].bytes);
            Launch(s, st);
            for (int id : {s.a, s.b})
                if (!persist_[id] && prefix_last_use_[id] == (int)i)
                    nodes_[id].own.reset(); // stream-ordered free
        }
        prefix_done_ = true;
    }

    void Launch(const Step &s, void *st, Profile *prof = nullptr)
    {
        const int dt = Gpu::DtypeCode<T>();
        const int idx = (int)(&s - steps_.data());
        const void *a = Buffer(s.a);
        const void *b = Buffer(s.b);
        // Steps that run once gain nothing from tuning: AUTO's rule.
        const int prec =
            (!s.chunk && precision_ == JETGPU_PREC_TUNED) ? JETGPU_PREC_AUTO : precision_;
        // Intermediates carry the max exponent their producing step recorded;
        // leaves are scanned when needed.
        int *emax = static_cast<int *>(emax_.get());
        const bool hints = exponent_hints_ && emax != nullptr;
        Gpu::Check(jetgpu_contract_batched_hinted(
                       s.batch, a, (int)s.a_shape.size(), s.a_shape.data(), s.a_perm.data(),
                       s.a_mode, b, (int)s.b_shape.size(), s.b_shape.data(), s.b_perm.data(),
                       s.b_mode, Buffer(s.out), s.m, s.n, s.k, dt, prec, JETGPU_ALGO_4M,
                       hints && s.a >= (int)num_leaves_ ? emax + s.a : nullptr,
                       hints && s.b >= (int)num_leaves_ ? emax + s.b : nullptr,
                       hints ? emax + s.out : nullptr, ws_.get(), ws_.size(), st),
                   "batched contraction");
        if (prof)
            prof->Mark("contract", idx, s.batch, s.m, s.n, s.k);
    }

    void Capture(void *st)
    {
        // One eager chunk first: first launches configure kernels (shared
        // memory limits, tensor-map encoder), which must not happen inside a
        // capture. Its effects (accumulator, counter) are undone below.
        uint64_t saved = 0;
        Gpu::Check(jetgpu_memcpy(&saved, counter_.get(), 8, 1, st), "counter read");
        Gpu::Synchronize();
        RecordChunk(st);
        Gpu::Check(jetgpu_memset_zero(acc_.get(), result_size_ * 16, st), "zero accumulator");
        Gpu::Check(jetgpu_memcpy(counter_.get(), &saved, 8, 0, st), "counter reset");
        Gpu::Synchronize();
        Gpu::Check(jetgpu_graph_begin(st), "capture begin");
        RecordChunk(st);
        Gpu::Check(jetgpu_graph_end(st, &graph_), "capture end");
    }

    // Enqueues one chunk: gather the "$s" leaves, run the "$s" steps, add the
    // chunk's slices into the FP64 accumulator, advance the slice counter.
    void RecordChunk(void *st, Profile *prof = nullptr)
    {
        const int dt = Gpu::DtypeCode<T>();
        for (const Loader &ld : loaders_) {
            Gpu::Check(jetgpu_slice_gather_at(leaves_[ld.leaf].GetDeviceData(),
                                              (int)ld.shape.size(), ld.shape.data(),
                                              (int)ld.axes.size(), ld.axes.data(),
                                              ld.value_strides.data(),
                                              static_cast<const uint64_t *>(counter_.get()),
                                              batch_, Buffer(ld.leaf), dt, st),
                       "slice gather");
            if (prof)
                prof->Mark("gather", -1, batch_, 0, 0, 0);
        }
        for (const Item &item : items_) {
            if (!item.grouped) {
                Launch(steps_[item.steps[0]], st, prof);
                continue;
            }
            Gpu::Check(jetgpu_contract_group(item.tasks, (int)item.steps.size(), item.tiles, dt,
                                             st),
                       "grouped contraction");
            if (prof)
                prof->Mark("group", item.steps.front(), item.steps.size(), 0, 0, 0);
        }
        const void *fin = Buffer(final_id_);
        if (final_perm_needed_) {
            Gpu::Check(jetgpu_permute(fin, final_tmp_.get(), (int)final_shape_.size(),
                                      final_shape_.data(), final_perm_.data(), dt, st),
                       "result reorder");
            fin = final_tmp_.get();
            if (prof)
                prof->Mark("result reorder", -1, batch_, 0, 0, 0);
        }
        Gpu::Check(jetgpu_slice_sum_f64(fin, batch_, result_size_, dt, acc_.get(), 1, st),
                   "slice sum");
        if (prof)
            prof->Mark("slice sum", -1, batch_, 0, 0, 0);
        Gpu::Check(jetgpu_counter_add(static_cast<uint64_t *>(counter_.get()), batch_, st),
                   "counter");
    }
};

} // namespace Jet
