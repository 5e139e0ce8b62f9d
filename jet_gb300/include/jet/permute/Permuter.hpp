// Jet::Permuter<Backend> (reference: include/jet/permute/Permuter.hpp:36-126),
// the permutation plugin point, with a GPU backend.
//
// The front-end validates exactly as the reference does and with the same
// messages (unique labels, matching shape/data sizes, a true permutation),
// then forwards to the backend. GpuPermuter moves the host data to the
// device, runs jetgpu_permute (one pass, bit-exact) and copies the result
// back; QFlexPermuter and DefaultPermuter run the same backend, so code
// written against the reference's backends compiles unchanged, and
// QFlexPermuter keeps the reference's acceptance rules (power-of-2 data, and
// the BLOCKSIZE / MIN_DIMS limits of its plan).
#pragma once

#include <algorithm>
#include <complex>
#include <unordered_map>
#include <set>
#include <string>
#include <type_traits>
#include <vector>

#include "../Abort.hpp"
#include "../Tensor.hpp"
#include "../Utilities.hpp"

namespace Jet {

class GpuPermuter {
  public:
    template <class DataType>
    void Transpose(const std::vector<DataType> &data_in, const std::vector<size_t> &shape,
                   std::vector<DataType> &data_out, const std::vector<std::string> &current,
                   const std::vector<std::string> &target)
    {
        static_assert(std::is_same_v<DataType, std::complex<float>> ||
                          std::is_same_v<DataType, std::complex<double>>,
                      "GpuPermuter permutes complex<float> or complex<double> data");
        data_out.resize(data_in.size());
        if (data_in.empty())
            return;
        std::vector<uint64_t> sh(shape.begin(), shape.end());
        std::vector<int32_t> perm(target.size());
        for (size_t j = 0; j < target.size(); ++j)
            perm[j] = (int32_t)(std::find(current.begin(), current.end(), target[j]) -
                                current.begin());
        const size_t bytes = data_in.size() * sizeof(DataType);
        Gpu::DeviceBuffer in(bytes), out(bytes);
        void *st = Gpu::Stream();
        Gpu::Check(jetgpu_memcpy(in.get(), data_in.data(), bytes, 0, st), "upload");
        Gpu::Check(jetgpu_permute(in.get(), out.get(), (int)sh.size(), sh.data(), perm.data(),
                                  Gpu::DtypeCode<DataType>(), st),
                   "permute");
        Gpu::Check(jetgpu_memcpy(data_out.data(), out.get(), bytes, 1, st), "download");
        Gpu::Synchronize();
    }

    template <class DataType>
    std::vector<DataType> Transpose(const std::vector<DataType> &data_in,
                                    const std::vector<size_t> &shape,
                                    const std::vector<std::string> &current,
                                    const std::vector<std::string> &target)
    {
        std::vector<DataType> out;
        Transpose(data_in, shape, out, current, target);
        return out;
    }
};

// QFlexPermuter<BLOCKSIZE, MIN_DIMS> (reference permute/QFlex.hpp:20-540): the
// GPU permutation behind the reference's acceptance rules. The reference
// plans a transpose of 2^n data over n binary indices in at most three
// passes split at BLOCKSIZE and MIN_DIMS, and rejects what that plan cannot
// express; CheckPlan restates the plan's decisions (not its data movement),
// so the same inputs are accepted and rejected with the same messages, and
// accepted inputs run as one bit-permutation pass on the device.
template <size_t BLOCKSIZE = 1024, size_t MIN_DIMS = 32> class QFlexPermuter : public GpuPermuter {
    static_assert(BLOCKSIZE > MIN_DIMS, "BLOCKSIZE must be greater than MIN_DIMS");

  public:
    template <class DataType>
    void Transpose(const std::vector<DataType> &data_in, const std::vector<size_t> &shape,
                   std::vector<DataType> &data_out, const std::vector<std::string> &current,
                   const std::vector<std::string> &target)
    {
        CheckPlan(shape, current, target);
        GpuPermuter::Transpose(data_in, shape, data_out, current, target);
    }

    template <class DataType>
    std::vector<DataType> Transpose(const std::vector<DataType> &data_in,
                                    const std::vector<size_t> &shape,
                                    const std::vector<std::string> &current,
                                    const std::vector<std::string> &target)
    {
        std::vector<DataType> out;
        Transpose(data_in, shape, out, current, target);
        return out;
    }

    // The reference plan's accept / reject decisions (QFlex.hpp:325-538).
    static void CheckPlan(const std::vector<size_t> &shape, const std::vector<std::string> &current,
                          const std::vector<std::string> &target)
    {
        using namespace Utilities;
        for (size_t d : shape)
            JET_ABORT_IF_NOT(d && !(d & (d - 1)), "Fast transpose expects power-of-2 data.");
        if (current == target)
            return;
        // One letter per binary index; an index of dimension 2^k owns k of them.
        std::unordered_map<std::string, std::vector<std::string>> groups;
        size_t letter = 0;
        for (size_t i = 0; i < current.size(); ++i) {
            std::vector<std::string> g;
            for (size_t d = shape[i]; d > 1; d >>= 1)
                g.push_back(GenerateStringIndex(letter++));
            groups.emplace(current[i], g);
        }
        std::vector<std::string> old_bin, new_bin;
        for (const auto &l : current)
            old_bin.insert(old_bin.end(), groups[l].begin(), groups[l].end());
        for (const auto &l : target)
            new_bin.insert(new_bin.end(), groups[l].begin(), groups[l].end());
        const size_t n = old_bin.size();
        const size_t lr = Log2(BLOCKSIZE), rr = Log2(MIN_DIMS);
        if (n <= lr)
            return; // one pass inside a block
        const size_t ll = n - lr;
        if (std::equal(old_bin.begin(), old_bin.begin() + ll, new_bin.begin()))
            return; // only the block-local part moves
        JET_ABORT_IF(rr == 0, "Number of minimum dimensions must be greater than one.");
        size_t suffix = 0;
        while (suffix < n && old_bin[n - 1 - suffix] == new_bin[n - 1 - suffix])
            ++suffix;
        if (suffix > 0 && suffix >= rr)
            return; // whole-chunk moves above a fixed suffix
        // Three-pass plan: its block-local step must hold every binary index
        // that ends up in the last rr positions.
        JET_ABORT_IF(n < rr, "New ordering is too small to be used at this point.");
        const size_t rl = n - rr;
        const std::vector<std::string> rr_new(new_bin.begin() + rl, new_bin.end());
        const std::vector<std::string> rl_old(old_bin.begin(), old_bin.begin() + rl);
        const auto moved = VectorIntersection(rl_old, rr_new);
        const auto first = VectorConcatenation(VectorSubtraction(rl_old, moved), moved);
        std::vector<std::string> lr_first(first.begin() + ll, first.end());
        lr_first.insert(lr_first.end(), old_bin.begin() + rl, old_bin.end());
        const auto lr_second = VectorConcatenation(VectorSubtraction(lr_first, rr_new), rr_new);
        JET_ABORT_IF(lr_second.size() != lr_first.size(),
                     "New ordering is too small to be used at this point. "
                     "Consider increasing the BLOCKSIZE.");
    }

  private:
    static constexpr size_t Log2(size_t v)
    {
        size_t r = 0;
        while (v > 1) {
            v >>= 1;
            ++r;
        }
        return r;
    }
};

// DefaultPermuter<BLOCKSIZE> (reference permute/Default.hpp:20-133): any
// dimensions; the same GPU permutation.
template <size_t BLOCKSIZE = 1024> class DefaultPermuter : public GpuPermuter {
};

template <class PermuterBackend> class Permuter {
  public:
    template <class DataType>
    void Transpose(const std::vector<DataType> &data_in, const std::vector<size_t> &shape,
                   std::vector<DataType> &data_out, const std::vector<std::string> &current_order,
                   const std::vector<std::string> &new_order)
    {
        Check(data_in, shape, current_order, new_order);
        JET_ABORT_IF_NOT(Utilities::ShapeToSize(shape) == data_out.size(),
                         "Tensor shape does not match given output tensor data.");
        backend_.Transpose(data_in, shape, data_out, current_order, new_order);
    }

    template <class DataType>
    std::vector<DataType> Transpose(const std::vector<DataType> &data_in,
                                    const std::vector<size_t> &shape,
                                    const std::vector<std::string> &current_order,
                                    const std::vector<std::string> &new_order)
    {
        Check(data_in, shape, current_order, new_order);
        JET_ABORT_IF(shape.empty(), "Tensor shape cannot be empty.");
        JET_ABORT_IF(new_order.empty(), "Tensor indices cannot be empty.");
        return backend_.Transpose(data_in, shape, current_order, new_order);
    }

  private:
    PermuterBackend backend_;

    template <class DataType>
    static void Check(const std::vector<DataType> &data_in, const std::vector<size_t> &shape,
                      const std::vector<std::string> &current, const std::vector<std::string> &target)
    {
        const std::set<std::string> old_set(current.begin(), current.end());
        const std::set<std::string> new_set(target.begin(), target.end());
        JET_ABORT_IF_NOT(old_set.size() == current.size(),
                         "Duplicate existing indices found. Please ensure indices are unique.");
        JET_ABORT_IF_NOT(new_set.size() == target.size(),
                         "Duplicate transpose indices found. Please ensure indices are unique.");
        JET_ABORT_IF_NOT(shape.size() == target.size(),
                         "Tensor shape does not match number of indices.");
        JET_ABORT_IF_NOT(Utilities::ShapeToSize(shape) == data_in.size(),
                         "Tensor shape does not match given tensor data.");
        JET_ABORT_IF_NOT(old_set == new_set,
                         "New indices are an invalid permutation of the existing indices");
    }
};

} // namespace Jet
