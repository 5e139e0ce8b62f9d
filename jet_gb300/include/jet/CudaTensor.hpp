// Jet::CudaTensor<T, CUDA_DEVICE> (reference: include/jet/CudaTensor.hpp:28-990),
// the reference's device-resident tensor type, served by the jetgpu kernels.
//
// Layout. The reference keeps a CudaTensor's data column-major over
// GetIndices() (the first index varies fastest; cuTENSOR modes). Column-major
// over labels L is row-major over reverse(L), so a CudaTensor here owns a
// Jet::Tensor with the reversed labels and shape on the same device buffer,
// and every operation maps onto the row-major kernels:
//   ContractTensors(a, b) = Tensor::ContractTensors(b', a'), whose labels
//       reverse(right) ++ reverse(left) are reverse(left ++ right);
//   Transpose(t, L)      = Tensor::Transpose(t', reverse(L));
//   SliceIndex, AddTensors, Reshape act on t' unchanged.
// Conversion to and from Jet::Tensor reverses labels and shape exactly as the
// reference does (:312-336, :400-410), so code that moves data between the two
// types keeps its meaning.
//
// The contraction plan (GetCudaContractionPlan / ContractTensorsWithoutAllocation,
// reference :470-669) holds the axis permutations, the m/n/k split and a
// preallocated workspace instead of a cuTENSOR plan; the product runs through
// jetgpu_contract (tcgen05 split precision or SIMT FP32 per
// Gpu::SetPrecision for complex64, FP64 for complex128).
//
// FillRandom draws re and im uniform in [0, 1) like the reference's
// curandGenerateUniform, from a seeded host generator (the values differ from
// cuRAND's; equal seeds give equal tensors).
#pragma once

#include <cuComplex.h>
#include <cuda_runtime_api.h>

#include <algorithm>
#include <complex>
#include <cstring>
#include <random>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "Abort.hpp"
#include "Tensor.hpp"
#include "Utilities.hpp"

namespace Jet {
namespace CudaTensorHelpers {

template <class T>
constexpr bool is_supported_data_type =
    std::is_same_v<T, cuComplex> || std::is_same_v<T, float2> ||
    std::is_same_v<T, cuDoubleComplex> || std::is_same_v<T, double2>;

template <class DataType>
static inline std::vector<DataType> ReverseVector(const std::vector<DataType> &input)
{
    return std::vector<DataType>{input.rbegin(), input.rend()};
}

// Selects `device` for the guard's scope and restores the previous device
// (reference CudaTensorHelpers.hpp:179-235).
class CudaScopedDevice {
  public:
    explicit CudaScopedDevice(int device)
    {
        Gpu::Check(jetgpu_get_device(&prev_device_), "CudaScopedDevice");
        if (prev_device_ == device)
            prev_device_ = -1;
        else
            Gpu::Check(jetgpu_set_device(device), "CudaScopedDevice");
    }
    ~CudaScopedDevice()
    {
        if (prev_device_ != -1)
            jetgpu_set_device(prev_device_);
    }
    CudaScopedDevice() = delete;
    CudaScopedDevice(const CudaScopedDevice &) = delete;
    CudaScopedDevice(CudaScopedDevice &&) = delete;

  private:
    int prev_device_ = -1;
};

} // namespace CudaTensorHelpers

template <class T = cuComplex, int CUDA_DEVICE = 0> class CudaTensor {
    static_assert(CudaTensorHelpers::is_supported_data_type<T>,
                  "CudaTensor supports cuComplex (float2) and cuDoubleComplex "
                  "(double2) data types.");

  public:
    using scalar_type_t = T;
    using scalar_type_t_precision = decltype(std::declval<T>().x);
    using host_type = std::complex<scalar_type_t_precision>;

    // ---- construction -----------------------------------------------------
    // One zero datum, no indices or shape (the reduction's zero sentinel).
    CudaTensor() { rm_ = Tensor<host_type>(); }

    CudaTensor(const std::vector<std::string> &indices, const std::vector<size_t> &shape)
    {
        InitIndicesAndShape(indices, shape);
    }

    CudaTensor(const std::vector<std::string> &indices, const std::vector<size_t> &shape,
               const std::vector<T> &data)
        : CudaTensor(indices, shape)
    {
        CopyHostDataToGpu(const_cast<T *>(data.data()));
    }

    CudaTensor(const std::vector<std::string> &indices, const std::vector<size_t> &shape,
               const T *data)
        : CudaTensor(indices, shape)
    {
        CopyHostDataToGpu(const_cast<T *>(data));
    }

    explicit CudaTensor(const std::vector<size_t> &shape)
    {
        std::vector<std::string> indices(shape.size());
        for (size_t i = 0; i < indices.size(); i++)
            indices[i] = std::string("?") + Utilities::GenerateStringIndex(i);
        InitIndicesAndShape(indices, shape);
    }

    CudaTensor(const CudaTensor &other) = default;
    CudaTensor(CudaTensor &&other) noexcept = default;
    CudaTensor &operator=(const CudaTensor &other) = default;
    CudaTensor &operator=(CudaTensor &&other) noexcept = default;

    // From a Jet::Tensor: labels and shape reversed, data unchanged.
    template <class CPUData> CudaTensor(const Tensor<CPUData> &other)
    {
        static_assert(sizeof(CPUData) == sizeof(T),
                      "Size of CPU and GPU data types do not match.");
        static_assert(std::is_same_v<CPUData, host_type>,
                      "CudaTensor<T> converts from Tensor<std::complex<T::x>>.");
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        SetLabels(CudaTensorHelpers::ReverseVector(other.GetIndices()),
                  CudaTensorHelpers::ReverseVector(other.GetShape()));
        rm_ = other;
    }

    template <class CPUData> CudaTensor &operator=(const Tensor<CPUData> &other)
    {
        *this = CudaTensor(other);
        return *this;
    }

    // To a Jet::Tensor: labels and shape reversed, data unchanged.
    explicit operator Tensor<host_type>() const { return rm_; }

    void InitIndicesAndShape(const std::vector<std::string> &indices,
                             const std::vector<size_t> &shape)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        SetLabels(indices, shape);
        rm_ = Tensor<host_type>(CudaTensorHelpers::ReverseVector(indices),
                                CudaTensorHelpers::ReverseVector(shape));
    }

    // ---- accessors --------------------------------------------------------
    const std::vector<std::string> &GetIndices() const { return indices_; }
    const std::vector<size_t> &GetShape() const { return shape_; }
    size_t GetSize() const { return Utilities::ShapeToSize(shape_); }
    const std::unordered_map<std::string, size_t> &GetIndexToDimension() const
    {
        return index_to_dimension_;
    }

    std::vector<size_t> ConvertIndicesToAxes(const std::vector<std::string> &indices) const
    {
        std::vector<size_t> axes(indices.size());
        for (size_t i = 0; i < indices.size(); i++)
            axes[i] = index_to_axes_.at(indices[i]);
        return axes;
    }

    // Device data (allocated on first use, under the tensor's device).
    T *GetData()
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        return reinterpret_cast<T *>(rm_.GetMutableDeviceData());
    }
    const T *GetData() const
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        return reinterpret_cast<const T *>(rm_.GetDeviceData());
    }

    void RenameIndex(size_t ind, std::string new_string)
    {
        const std::string old_string = indices_[ind];
        if (old_string == new_string)
            return;
        JET_ABORT_IF_NOT(index_to_dimension_.find(new_string) == index_to_dimension_.end(),
                         "Renaming index to already existing value is not allowed.");
        indices_[ind] = new_string;
        index_to_dimension_[new_string] = index_to_dimension_[old_string];
        index_to_dimension_.erase(old_string);
        index_to_axes_[new_string] = ind;
        index_to_axes_.erase(old_string);
        rm_.RenameIndex(indices_.size() - 1 - ind, new_string);
    }

    // ---- host <-> device copies -------------------------------------------
    void CopyHostDataToGpu(T *host_tensor)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        Gpu::Check(jetgpu_memcpy(GetData(), host_tensor, Bytes(), 0, Gpu::Stream()),
                   "CopyHostDataToGpu");
        Gpu::Synchronize();
    }

    void CopyGpuDataToHost(T *host_tensor) const
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        Gpu::Check(jetgpu_memcpy(host_tensor, GetData(), Bytes(), 1, Gpu::Stream()),
                   "CopyGpuDataToHost");
        Gpu::Synchronize();
    }

    // Copies this tensor's data to the device buffer `dst`.
    void CopyGpuDataToGpu(T *dst)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        Gpu::Check(jetgpu_memcpy(dst, GetData(), Bytes(), 2, Gpu::Stream()), "CopyGpuDataToGpu");
        Gpu::Synchronize();
    }

    void AsyncCopyHostDataToGpu(T *host_tensor, cudaStream_t stream = 0)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        T *dst = GetData();
        Gpu::Synchronize(); // library-stream work on this tensor precedes `stream`
        Gpu::Check(jetgpu_memcpy(dst, host_tensor, Bytes(), 0, StreamOf(stream)),
                   "AsyncCopyHostDataToGpu");
    }

    void AsyncCopyGpuDataToHost(T *host_tensor, cudaStream_t stream = 0)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(CUDA_DEVICE);
        const T *src = GetData();
        Gpu::Synchronize();
        Gpu::Check(jetgpu_memcpy(host_tensor, src, Bytes(), 1, StreamOf(stream)),
                   "AsyncCopyGpuDataToHost");
    }

    std::vector<host_type> GetHostDataVector() const
    {
        std::vector<host_type> host(GetSize());
        CopyGpuDataToHost(reinterpret_cast<T *>(host.data()));
        return host;
    }

    void FillRandom(size_t seed)
    {
        std::mt19937_64 engine(seed);
        Fill(engine);
    }

    void FillRandom()
    {
        static std::mt19937_64 engine(std::random_device{}());
        Fill(engine);
    }

    // ---- contraction --------------------------------------------------------
    // Axis permutations, m/n/k and workspace of one contraction C = A . B, in
    // the row-major (reversed-label) frame where A' = b and B' = a.
    struct CudaContractionPlan {
        std::vector<uint64_t> x_shape, y_shape, c_tmp_shape;
        std::vector<int32_t> x_perm, y_perm, c_perm;
        uint64_t m = 1, n = 1, k = 1;
        int precision = JETGPU_PREC_FP32;
        bool permute_out = false; // C's label order differs from left ++ right
        size_t work_size = 0;
        Gpu::DeviceBuffer work;
    };

    template <class U = T, int D = CUDA_DEVICE>
    static void GetCudaContractionPlan(CudaContractionPlan &cplan, const CudaTensor<U, D> &a_tensor,
                                       const CudaTensor<U, D> &b_tensor,
                                       const CudaTensor<U, D> &c_tensor)
    {
        using namespace Utilities;
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        const auto &x = b_tensor.rm_; // row-major frame: C' = b' . a'
        const auto &y = a_tensor.rm_;
        const auto left = VectorSubtraction(x.GetIndices(), y.GetIndices());
        const auto right = VectorSubtraction(y.GetIndices(), x.GetIndices());
        const auto common = VectorIntersection(x.GetIndices(), y.GetIndices());
        const auto &xd = x.GetIndexToDimension();
        const auto &yd = y.GetIndexToDimension();
        cplan.m = cplan.n = cplan.k = 1;
        cplan.x_perm.clear();
        cplan.y_perm.clear();
        cplan.c_tmp_shape.clear();
        for (const auto &l : left) {
            cplan.m *= xd.at(l);
            cplan.c_tmp_shape.push_back(xd.at(l));
        }
        for (const auto &l : right) {
            cplan.n *= yd.at(l);
            cplan.c_tmp_shape.push_back(yd.at(l));
        }
        for (const auto &l : common)
            cplan.k *= xd.at(l);
        for (const auto &l : VectorConcatenation(left, common))
            cplan.x_perm.push_back((int32_t)Position(x.GetIndices(), l));
        for (const auto &l : VectorConcatenation(common, right))
            cplan.y_perm.push_back((int32_t)Position(y.GetIndices(), l));
        cplan.x_shape.assign(x.GetShape().begin(), x.GetShape().end());
        cplan.y_shape.assign(y.GetShape().begin(), y.GetShape().end());
        // C's row-major labels must be a permutation of left ++ right.
        const auto tmp_labels = VectorConcatenation(left, right);
        const auto &c_labels = c_tensor.rm_.GetIndices();
        JET_ABORT_IF_NOT(c_labels.size() == tmp_labels.size() &&
                             VectorDisjunctiveUnion(c_labels, tmp_labels).empty(),
                         "Output tensor indices do not match the contraction.");
        cplan.permute_out = c_labels != tmp_labels;
        cplan.c_perm.clear();
        for (const auto &l : c_labels)
            cplan.c_perm.push_back((int32_t)Position(tmp_labels, l));
        const int dt = DtypeOf<U>();
        cplan.precision = dt == JETGPU_C128 ? JETGPU_PREC_FP32 : Gpu::GetPrecision();
        size_t ws = jetgpu_contract_workspace_size(
            (int)cplan.x_shape.size(), cplan.x_shape.data(), cplan.x_perm.data(),
            (int)cplan.y_shape.size(), cplan.y_shape.data(), cplan.y_perm.data(), cplan.m,
            cplan.n, cplan.k, dt, cplan.precision);
        ws = (ws + 255) / 256 * 256;
        if (cplan.permute_out)
            ws += cplan.m * cplan.n * sizeof(U);
        cplan.work_size = ws;
        cplan.work = Gpu::DeviceBuffer(ws);
    }

    // C = A . B into the preallocated `c` with a plan from GetCudaContractionPlan;
    // enqueued on `stream` (0: the library stream), no allocation.
    template <class U = T, int D = CUDA_DEVICE>
    static void ContractTensorsWithoutAllocation(const CudaTensor<U, D> &a,
                                                 const CudaTensor<U, D> &b, CudaTensor<U, D> &c,
                                                 CudaContractionPlan &c_plan,
                                                 cudaStream_t stream = 0)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        const void *x = b.GetData();
        const void *y = a.GetData();
        void *out = c.GetData();
        if (stream != 0)
            Gpu::Synchronize(); // operands written on the library stream
        void *st = StreamOf(stream);
        const int dt = DtypeOf<U>();
        uint8_t *work = static_cast<uint8_t *>(c_plan.work.get());
        size_t work_bytes = c_plan.work_size;
        void *dst = out;
        if (c_plan.permute_out) {
            const size_t tmp_bytes = c_plan.m * c_plan.n * sizeof(U);
            work_bytes -= tmp_bytes;
            dst = work + work_bytes;
        }
        Gpu::Check(jetgpu_contract(x, (int)c_plan.x_shape.size(), c_plan.x_shape.data(),
                                   c_plan.x_perm.data(), y, (int)c_plan.y_shape.size(),
                                   c_plan.y_shape.data(), c_plan.y_perm.data(), dst, c_plan.m,
                                   c_plan.n, c_plan.k, dt, c_plan.precision, JETGPU_ALGO_4M, 0, 0,
                                   work_bytes ? work : nullptr, work_bytes, st),
                   "ContractTensorsWithoutAllocation");
        if (c_plan.permute_out)
            Gpu::Check(jetgpu_permute(dst, out, (int)c_plan.c_tmp_shape.size(),
                                      c_plan.c_tmp_shape.data(), c_plan.c_perm.data(), dt, st),
                       "ContractTensorsWithoutAllocation");
    }

    template <class U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> ContractTensors(const CudaTensor<U, D> &a_tensor,
                                            const CudaTensor<U, D> &b_tensor)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        CudaTensor<U, D> c;
        c.rm_ = Tensor<host_type>::ContractTensors(b_tensor.rm_, a_tensor.rm_);
        c.SetLabels(CudaTensorHelpers::ReverseVector(c.rm_.GetIndices()),
                    CudaTensorHelpers::ReverseVector(c.rm_.GetShape()));
        return c;
    }

    CudaTensor<T, CUDA_DEVICE> ContractTensors(const CudaTensor<T, CUDA_DEVICE> &other) const
    {
        return ContractTensors<T, CUDA_DEVICE>(*this, other);
    }

    // ---- other operations -------------------------------------------------
    template <class U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> AddTensors(const CudaTensor<U, D> &A, const CudaTensor<U, D> &B)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        CudaTensor<U, D> C;
        C.rm_ = Tensor<host_type>::AddTensors(A.rm_, B.rm_);
        C.SetLabels(CudaTensorHelpers::ReverseVector(C.rm_.GetIndices()),
                    CudaTensorHelpers::ReverseVector(C.rm_.GetShape()));
        return C;
    }

    CudaTensor<T, CUDA_DEVICE> AddTensor(const CudaTensor<T, CUDA_DEVICE> &other) const
    {
        return AddTensors<T, CUDA_DEVICE>(*this, other);
    }

    template <typename U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> Reshape(const CudaTensor<U, D> &old_tensor,
                                    const std::vector<size_t> &new_shape)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        JET_ABORT_IF_NOT(old_tensor.GetSize() == Utilities::ShapeToSize(new_shape),
                         "Size is inconsistent between tensors.");
        CudaTensor<U, D> reshaped(new_shape);
        Gpu::Check(jetgpu_memcpy(reshaped.GetData(), old_tensor.GetData(),
                                 sizeof(U) * old_tensor.GetSize(), 2, Gpu::Stream()),
                   "Reshape");
        return reshaped;
    }

    CudaTensor<T, CUDA_DEVICE> Reshape(const std::vector<size_t> &new_shape)
    {
        return Reshape<T, CUDA_DEVICE>(*this, new_shape);
    }

    template <class U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> Transpose(const CudaTensor<U, D> &tensor,
                                      const std::vector<std::string> &new_indices)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        if (tensor.GetIndices() == new_indices)
            return tensor;
        JET_ABORT_IF(tensor.GetIndices().empty(), "Number of indices cannot be zero.");
        CudaTensor<U, D> out;
        out.rm_ = Tensor<host_type>::Transpose(tensor.rm_,
                                               CudaTensorHelpers::ReverseVector(new_indices));
        out.SetLabels(new_indices, CudaTensorHelpers::ReverseVector(out.rm_.GetShape()));
        return out;
    }

    template <class U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> Transpose(const CudaTensor<U, D> &A,
                                      const std::vector<size_t> &new_ordering)
    {
        const size_t num_indices = A.GetIndices().size();
        JET_ABORT_IF_NOT(num_indices == new_ordering.size(),
                         "Size of ordering must match number of tensor indices.");
        std::vector<std::string> new_indices(num_indices);
        for (size_t i = 0; i < num_indices; i++)
            new_indices[i] = A.GetIndices()[new_ordering[i]];
        return Transpose<U, D>(A, new_indices);
    }

    CudaTensor<T, CUDA_DEVICE> Transpose(const std::vector<size_t> &new_ordering) const
    {
        return Transpose<T, CUDA_DEVICE>(*this, new_ordering);
    }

    CudaTensor<T, CUDA_DEVICE> Transpose(const std::vector<std::string> &new_indices) const
    {
        return Transpose<T, CUDA_DEVICE>(*this, new_indices);
    }

    template <typename U = T, int D = CUDA_DEVICE>
    static CudaTensor<U, D> SliceIndex(const CudaTensor<U, D> &tens, const std::string &index_str,
                                       size_t index_value)
    {
        CudaTensorHelpers::CudaScopedDevice ctx(D);
        CudaTensor<U, D> out;
        out.rm_ = Tensor<host_type>::SliceIndex(tens.rm_, index_str, index_value);
        out.SetLabels(CudaTensorHelpers::ReverseVector(out.rm_.GetIndices()),
                      CudaTensorHelpers::ReverseVector(out.rm_.GetShape()));
        return out;
    }

    CudaTensor<T, CUDA_DEVICE> SliceIndex(const std::string &index_str, size_t index_value)
    {
        return SliceIndex<T, CUDA_DEVICE>(*this, index_str, index_value);
    }

    bool operator==(const CudaTensor<T, CUDA_DEVICE> &other) const
    {
        return shape_ == other.GetShape() && indices_ == other.GetIndices() &&
               index_to_dimension_ == other.GetIndexToDimension() &&
               GetHostDataVector() == other.GetHostDataVector();
    }

  private:
    template <class, int> friend class CudaTensor;

    Tensor<host_type> rm_; // row-major over reversed labels, same buffer
    std::vector<std::string> indices_;
    std::vector<size_t> shape_;
    std::unordered_map<std::string, size_t> index_to_dimension_;
    std::unordered_map<std::string, size_t> index_to_axes_;

    void SetLabels(const std::vector<std::string> &indices, const std::vector<size_t> &shape)
    {
        indices_ = indices;
        shape_ = shape;
        index_to_dimension_.clear();
        index_to_axes_.clear();
        for (size_t i = 0; i < shape_.size(); ++i) {
            index_to_dimension_[indices_[i]] = shape_[i];
            index_to_axes_[indices_[i]] = i;
        }
    }

    size_t Bytes() const { return sizeof(T) * GetSize(); }

    static size_t Position(const std::vector<std::string> &v, const std::string &x)
    {
        return static_cast<size_t>(std::find(v.begin(), v.end(), x) - v.begin());
    }

    template <class U> static constexpr int DtypeOf()
    {
        return (std::is_same_v<U, cuDoubleComplex> || std::is_same_v<U, double2>) ? JETGPU_C128
                                                                                    : JETGPU_C64;
    }

    static void *StreamOf(cudaStream_t stream)
    {
        return stream ? reinterpret_cast<void *>(stream) : Gpu::Stream();
    }

    template <class Engine> void Fill(Engine &engine)
    {
        std::uniform_real_distribution<scalar_type_t_precision> dist(0, 1);
        std::vector<host_type> host(GetSize());
        for (auto &v : host) {
            const auto re = dist(engine);
            const auto im = dist(engine);
            v = {re, im};
        }
        CopyHostDataToGpu(reinterpret_cast<T *>(host.data()));
    }
};

} // namespace Jet
