// Jet::Permuter<Backend> (reference: include/jet/permute/Permuter.hpp:36-126),
// the permutation plugin point, with a GPU backend.
//
// The front-end validates exactly as the reference does and with the same
// messages (unique labels, matching shape/data sizes, a true permutation),
// then forwards to the backend. GpuPermuter moves the host data to the
// device, runs jetgpu_permute (one pass, bit-exact) and copies the result
// back; QFlexPermuter and DefaultPermuter name the same backend here, so code
// written against the reference's backends compiles unchanged (the BLOCKSIZE
// and MIN_DIMS parameters only tuned the CPU algorithms).
#pragma once

#include <complex>
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

template <size_t BLOCKSIZE = 1024, size_t MIN_DIMS = 32> class QFlexPermuter : public GpuPermuter {
};
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
