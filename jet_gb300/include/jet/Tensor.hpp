// Jet::Tensor on a GB300: the reference's tensor API (include/jet/Tensor.hpp)
// with device-resident data.
//
// The data live in device memory (jetgpu_malloc, stream-ordered on the library
// stream) and are mirrored on the host only when host code reads or writes
// them: GetData(), operator[], GetValue() download on demand; SetData(),
// SetValue(), FillRandom() and the non-const accessors update the host copy
// and invalidate the device copy, which is uploaded again at the next device
// operation. ContractTensors, Transpose, SliceIndex, AddTensors, Reshape and
// Conj run as CUDA kernels through the C-ABI in jetgpu.h and never touch the
// host data. Labels, shapes and the label algebra stay on the host and follow
// the reference exactly, so results carry the same index order.
//
// Arithmetic form of ContractTensors (complex64): Gpu::SetPrecision(
// JETGPU_PREC_FP32 | JETGPU_PREC_TF32X3 | JETGPU_PREC_AUTO | JETGPU_PREC_BF16X3 |
// JETGPU_PREC_FP16X3 | JETGPU_PREC_TUNED);
// default FP32, the arithmetic class of the reference's cgemm. complex128
// always uses FP64.
#pragma once

#include <algorithm>
#include <atomic>
#include <complex>
#include <cstring>
#include <iostream>
#include <mutex>
#include <random>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "jetgpu.h"

#include "Abort.hpp"
#include "Utilities.hpp"

namespace Jet {
namespace Gpu {

inline std::atomic<int> &PrecisionSetting()
{
    static std::atomic<int> p{JETGPU_PREC_FP32};
    return p;
}
inline void SetPrecision(int precision) { PrecisionSetting().store(precision); }
inline int GetPrecision() { return PrecisionSetting().load(); }

inline void Check(int rc, const char *what)
{
    if (rc != JETGPU_OK)
        JET_ABORT(std::string(what) + ": " + jetgpu_last_error());
}

inline void *Stream() { return jetgpu_default_stream(); }

inline void Synchronize() { Check(jetgpu_stream_synchronize(Stream()), "synchronize"); }

// A named NVTX range over the scope (jetgpu_range_push / jetgpu_range_pop):
// the host loops show up in a timeline around the library's own ranges.
class Range {
  public:
    explicit Range(const char *name) { jetgpu_range_push(name); }
    ~Range() { jetgpu_range_pop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

// Device time of consecutive stretches of work on a stream: each Mark()
// records a CUDA event; Finish() waits and returns the ms between each mark
// and the one before (the first against construction).
class StreamTimer {
  public:
    explicit StreamTimer(void *stream) : stream_(stream) { Push(); }
    ~StreamTimer()
    {
        for (void *e : events_)
            jetgpu_event_destroy(e);
    }
    StreamTimer(const StreamTimer &) = delete;
    StreamTimer &operator=(const StreamTimer &) = delete;
    void Mark() { Push(); }
    std::vector<double> Finish()
    {
        std::vector<double> ms;
        for (size_t i = 1; i < events_.size(); ++i) {
            float t = 0;
            Check(jetgpu_event_elapsed_ms(events_[i - 1], events_[i], &t), "event time");
            ms.push_back(t);
        }
        return ms;
    }

  private:
    void Push()
    {
        void *e = nullptr;
        Check(jetgpu_event_create(&e), "event create");
        events_.push_back(e);
        Check(jetgpu_event_record(e, stream_), "event record");
    }
    void *stream_;
    std::vector<void *> events_;
};

// Move-only owner of a device allocation from the library allocator.
class DeviceBuffer {
  public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t bytes) : bytes_(bytes)
    {
        if (bytes)
            Check(jetgpu_malloc(bytes, &ptr_), "jetgpu_malloc");
    }
    DeviceBuffer(const DeviceBuffer &) = delete;
    DeviceBuffer &operator=(const DeviceBuffer &) = delete;
    DeviceBuffer(DeviceBuffer &&o) noexcept : ptr_(o.ptr_), bytes_(o.bytes_)
    {
        o.ptr_ = nullptr;
        o.bytes_ = 0;
    }
    DeviceBuffer &operator=(DeviceBuffer &&o) noexcept
    {
        if (this != &o) {
            reset();
            ptr_ = o.ptr_;
            bytes_ = o.bytes_;
            o.ptr_ = nullptr;
            o.bytes_ = 0;
        }
        return *this;
    }
    ~DeviceBuffer() { reset(); }
    void reset()
    {
        if (ptr_)
            jetgpu_free(ptr_);
        ptr_ = nullptr;
        bytes_ = 0;
    }
    void *get() const { return ptr_; }
    size_t size() const { return bytes_; }

  private:
    void *ptr_ = nullptr;
    size_t bytes_ = 0;
};

template <class T> constexpr int DtypeCode()
{
    return std::is_same_v<T, std::complex<double>> ? JETGPU_C128 : JETGPU_C64;
}

} // namespace Gpu

template <class T = std::complex<float>> class Tensor {
    static_assert(std::is_same_v<T, std::complex<float>> ||
                      std::is_same_v<T, std::complex<double>>,
                  "Tensor data type must be one of std::complex<float>, "
                  "std::complex<double>");

  public:
    using scalar_type_t = T;

    // One zero datum, no indices or shape (the reduction's zero sentinel).
    Tensor() : size_(1), host_(1, T{0}), host_valid_(true) {}

    explicit Tensor(const std::vector<size_t> &shape) : size_(Utilities::ShapeToSize(shape))
    {
        std::vector<std::string> labels(shape.size());
        for (size_t i = 0; i < shape.size(); ++i)
            labels[i] = "?" + Utilities::GenerateStringIndex(i);
        InitIndicesAndShape(labels, shape);
    }

    Tensor(const std::vector<std::string> &indices, const std::vector<size_t> &shape)
        : size_(Utilities::ShapeToSize(shape))
    {
        InitIndicesAndShape(indices, shape);
    }

    Tensor(const std::vector<std::string> &indices, const std::vector<size_t> &shape,
           const std::vector<T> &data)
        : Tensor(indices, shape)
    {
        host_ = data;
        host_.resize(size_);
        host_valid_ = true;
    }

    Tensor(const Tensor &other) { CopyFrom(other); }

    Tensor(Tensor &&other) noexcept { MoveFrom(std::move(other)); }

    virtual ~Tensor() = default;

    const Tensor &operator=(const Tensor &other)
    {
        if (this != &other)
            CopyFrom(other);
        return *this;
    }

    const Tensor &operator=(Tensor &&other) noexcept
    {
        if (this != &other)
            MoveFrom(std::move(other));
        return *this;
    }

    // The label -> dimension map is built from the labels and shape when it
    // is first read (GetIndexToDimension, RenameIndex, ==), by the same rule
    // as the reference's constructor: a contraction step creates a tensor
    // whose map nothing reads (building it cost about 1 us of host time for
    // a rank-27 result).
    void InitIndicesAndShape(const std::vector<std::string> &indices,
                             const std::vector<size_t> &shape) noexcept
    {
        indices_ = indices;
        shape_ = shape;
        index_to_dimension_.clear();
        dims_built_ = false;
    }

    // As the reference's SetShape, the map keeps the dimensions it had.
    void SetShape(const std::vector<size_t> &shape) noexcept
    {
        GetIndexToDimension();
        shape_ = shape;
    }
    const std::vector<size_t> &GetShape() const noexcept { return shape_; }
    const std::vector<std::string> &GetIndices() const noexcept { return indices_; }
    const std::unordered_map<std::string, size_t> &GetIndexToDimension() const
    {
        std::lock_guard<std::mutex> lock(sync_);
        if (!dims_built_) {
            for (size_t i = 0; i < shape_.size(); ++i)
                index_to_dimension_[indices_[i]] = shape_[i];
            dims_built_ = true;
        }
        return index_to_dimension_;
    }

    void RenameIndex(size_t pos, std::string new_label) noexcept
    {
        GetIndexToDimension();
        const auto old = indices_[pos];
        const size_t dim = index_to_dimension_[old];
        index_to_dimension_.erase(old);
        indices_[pos] = new_label;
        index_to_dimension_.emplace(new_label, dim);
    }

    T &operator[](size_t pos) { return HostMutable()[pos]; }
    const T &operator[](size_t pos) const { return HostView()[pos]; }

    bool operator==(const Tensor &other) const
    {
        return shape_ == other.shape_ && indices_ == other.indices_ &&
               GetIndexToDimension() == other.GetIndexToDimension() &&
               HostView() == other.HostView();
    }
    bool operator!=(const Tensor &other) const { return !(*this == other); }

    void SetValue(const std::vector<size_t> &idx, const T &value)
    {
        HostMutable()[Utilities::RavelIndex(idx, shape_)] = value;
    }
    T GetValue(const std::vector<size_t> &idx) const
    {
        return HostView()[Utilities::RavelIndex(idx, shape_)];
    }

    void SetData(const std::vector<T> &data)
    {
        JET_ABORT_IF_NOT(data.size() == GetSize(), "Size of data and tensor do not match.");
        host_ = data;
        host_valid_ = true;
        dev_valid_ = false;
    }

    const std::vector<T> &GetData() const { return HostView(); }
    std::vector<T> &GetData() { return HostMutable(); }

    size_t GetSize() const { return size_; }
    const T &GetScalar() const { return HostView()[0]; }
    bool IsScalar() const noexcept { return size_ == 1; }

    // Same engine and distribution as the reference (Tensor.hpp:361-369).
    void FillRandom(size_t seed)
    {
        std::mt19937 engine(seed);
        std::uniform_real_distribution<typename T::value_type> dist(-1, 1);
        auto &d = HostMutable();
        for (size_t i = 0; i < size_; ++i) {
            const auto re = dist(engine);
            const auto im = dist(engine);
            d[i] = {re, im};
        }
    }

    void FillRandom()
    {
        static std::mt19937 engine(std::random_device{}());
        std::uniform_real_distribution<typename T::value_type> dist(-1, 1);
        auto &d = HostMutable();
        for (size_t i = 0; i < size_; ++i) {
            const auto re = dist(engine);
            const auto im = dist(engine);
            d[i] = {re, im};
        }
    }

    // ---- device access ------------------------------------------------------
    const T *GetDeviceData() const
    {
        SyncDevice();
        return static_cast<const T *>(dev_.get());
    }
    T *GetMutableDeviceData()
    {
        SyncDevice();
        host_valid_ = false;
        return static_cast<T *>(dev_.get());
    }
    // Copies `size` elements from a device pointer into this tensor.
    void SetDeviceData(const T *src)
    {
        AllocateDevice();
        Gpu::Check(jetgpu_memcpy(dev_.get(), src, size_ * sizeof(T), 2, Gpu::Stream()),
                   "SetDeviceData");
        dev_valid_ = true;
        host_valid_ = false;
    }

    // ---- static operations (device kernels) ----------------------------------
    template <class U = T> static Tensor<U> AddTensors(const Tensor<U> &A, const Tensor<U> &B)
    {
        if (A.IsZeroSentinel())
            return B;
        if (B.IsZeroSentinel())
            return A;
        JET_ABORT_IF_NOT(
            Utilities::VectorDisjunctiveUnion(A.GetIndices(), B.GetIndices()).empty(),
            "Tensor addition with disjoint indices is not supported.");
        const Tensor<U> Bt = Transpose(B, A.GetIndices());
        Tensor<U> C(A.GetIndices(), A.GetShape());
        C.AllocateDevice();
        Gpu::Check(jetgpu_add(A.GetDeviceData(), Bt.GetDeviceData(), C.dev_.get(), C.size_,
                              Gpu::DtypeCode<U>(), Gpu::Stream()),
                   "AddTensors");
        C.MarkDeviceWritten();
        return C;
    }
    Tensor<T> AddTensor(const Tensor<T> &other) const { return AddTensors<T>(*this, other); }

    template <class U = T>
    static Tensor<U> SliceIndex(const Tensor<U> &tensor, const std::string &index, size_t value)
    {
        const auto &lab = tensor.GetIndices();
        const auto it = std::find(lab.begin(), lab.end(), index);
        JET_ABORT_IF(it == lab.end(), "Sliced index does not exist.");
        const int32_t axis = static_cast<int32_t>(it - lab.begin());
        std::vector<std::string> rest;
        std::vector<size_t> rest_shape;
        for (size_t i = 0; i < lab.size(); ++i)
            if ((int32_t)i != axis) {
                rest.push_back(lab[i]);
                rest_shape.push_back(tensor.GetShape()[i]);
            }
        JET_ABORT_IF(value >= tensor.GetShape()[axis], "Slice value out of range.");
        Tensor<U> out(rest, rest_shape);
        out.AllocateDevice();
        std::vector<uint64_t> shape(tensor.GetShape().begin(), tensor.GetShape().end());
        const uint64_t stride = 1;
        Gpu::Check(jetgpu_slice_gather(tensor.GetDeviceData(), (int)shape.size(), shape.data(),
                                       1, &axis, &stride, value, 1, out.dev_.get(),
                                       Gpu::DtypeCode<U>(), Gpu::Stream()),
                   "SliceIndex");
        out.MarkDeviceWritten();
        return out;
    }
    Tensor<T> SliceIndex(const std::string &index, size_t value) const
    {
        return SliceIndex<T>(*this, index, value);
    }

    template <class U = T>
    static Tensor<U> Reshape(const Tensor<U> &old_tensor, const std::vector<size_t> &new_shape)
    {
        JET_ABORT_IF_NOT(old_tensor.GetSize() == Utilities::ShapeToSize(new_shape),
                         "Size is inconsistent between tensors.");
        Tensor<U> t(new_shape);
        t.CopyDataFrom(old_tensor);
        return t;
    }
    Tensor<T> Reshape(const std::vector<size_t> &new_shape) const
    {
        return Reshape<T>(*this, new_shape);
    }

    template <class U = T>
    static Tensor<U> Transpose(const Tensor<U> &A, const std::vector<std::string> &new_indices)
    {
        if (A.GetIndices() == new_indices)
            return A;
        if (A.GetIndices().empty())
            JET_ABORT("Number of indices cannot be zero.");
        ValidateOrdering(A.GetIndices(), new_indices);
        std::vector<size_t> new_shape(new_indices.size());
        std::vector<int32_t> perm(new_indices.size());
        for (size_t j = 0; j < new_indices.size(); ++j) {
            new_shape[j] = A.GetIndexToDimension().at(new_indices[j]);
            perm[j] = static_cast<int32_t>(
                std::find(A.GetIndices().begin(), A.GetIndices().end(), new_indices[j]) -
                A.GetIndices().begin());
        }
        Tensor<U> out(new_indices, new_shape);
        out.AllocateDevice();
        std::vector<uint64_t> shape(A.GetShape().begin(), A.GetShape().end());
        Gpu::Check(jetgpu_permute(A.GetDeviceData(), out.dev_.get(), (int)shape.size(),
                                  shape.data(), perm.data(), Gpu::DtypeCode<U>(), Gpu::Stream()),
                   "Transpose");
        out.MarkDeviceWritten();
        return out;
    }

    template <class U = T>
    static Tensor<U> Transpose(const Tensor<U> &A, const std::vector<size_t> &new_ordering)
    {
        const size_t n = A.GetIndices().size();
        JET_ABORT_IF_NOT(n == new_ordering.size(),
                         "Size of ordering must match number of tensor indices.");
        std::vector<std::string> labels(n);
        for (size_t i = 0; i < n; ++i)
            labels[i] = A.GetIndices()[new_ordering[i]];
        return Transpose<U>(A, labels);
    }
    Tensor<T> Transpose(const std::vector<size_t> &new_ordering) const
    {
        return Transpose<T>(*this, new_ordering);
    }
    Tensor<T> Transpose(const std::vector<std::string> &new_indices) const
    {
        return Transpose<T>(*this, new_indices);
    }

    template <class U = T> static Tensor<U> Conj(const Tensor<U> &A)
    {
        Tensor<U> out(A.GetIndices(), A.GetShape());
        out.AllocateDevice();
        Gpu::Check(jetgpu_conj(A.GetDeviceData(), out.dev_.get(), A.GetSize(),
                               Gpu::DtypeCode<U>(), Gpu::Stream()),
                   "Conj");
        out.MarkDeviceWritten();
        return out;
    }
    Tensor<T> Conj() const { return Conj<T>(*this); }

    // The device call of one pairwise contraction, from the operands' labels
    // and shapes: labels left = A\B (A order), right = B\A (B order),
    // common = A∩B (A order); C carries left ++ right; a_perm / b_perm order
    // A as (left ++ common) and B as (common ++ right).
    struct ContractionLayout {
        std::vector<std::string> c_indices;
        std::vector<size_t> c_shape;
        std::vector<uint64_t> a_shape, b_shape;
        std::vector<int32_t> a_perm, b_perm;
        uint64_t m = 1, n = 1, k = 1;
    };
    // One pass over the label pairs (ranks are at most 64): the same sets as
    // VectorSubtraction / VectorIntersection (Utilities.hpp) build through
    // hash sets, without their allocations -- this runs once per path step.
    template <class U = T>
    static ContractionLayout LayoutOf(const Tensor<U> &A, const Tensor<U> &B)
    {
        ContractionLayout l;
        const auto &ai = A.GetIndices();
        const auto &bi = B.GetIndices();
        const auto &as = A.GetShape();
        const auto &bs = B.GetShape();
        const size_t ra = ai.size(), rb = bi.size();
        std::vector<int32_t> b_pos(ra, -1); // first position in B of A's label i
        std::vector<char> b_in_a(rb, 0);
        for (size_t i = 0; i < ra; ++i)
            for (size_t j = 0; j < rb; ++j)
                if (ai[i] == bi[j]) {
                    if (b_pos[i] < 0)
                        b_pos[i] = static_cast<int32_t>(j);
                    b_in_a[j] = 1;
                }
        l.c_indices.reserve(ra + rb);
        l.c_shape.reserve(ra + rb);
        l.a_perm.reserve(ra);
        l.b_perm.reserve(rb);
        for (size_t i = 0; i < ra; ++i)
            if (b_pos[i] < 0) { // left = A \ B
                l.m *= as[i];
                l.c_shape.push_back(as[i]);
                l.c_indices.push_back(ai[i]);
                l.a_perm.push_back(static_cast<int32_t>(i));
            }
        for (size_t i = 0; i < ra; ++i)
            if (b_pos[i] >= 0) { // common = A ∩ B, in A's order
                l.k *= as[i];
                l.a_perm.push_back(static_cast<int32_t>(i));
                l.b_perm.push_back(b_pos[i]);
            }
        for (size_t j = 0; j < rb; ++j)
            if (!b_in_a[j]) { // right = B \ A
                l.n *= bs[j];
                l.c_shape.push_back(bs[j]);
                l.c_indices.push_back(bi[j]);
                l.b_perm.push_back(static_cast<int32_t>(j));
            }
        l.a_shape.assign(as.begin(), as.end());
        l.b_shape.assign(bs.begin(), bs.end());
        return l;
    }

    // Precision a contraction of this element type runs in: the setting for
    // complex64, FP64 for complex128.
    template <class U = T> static int ContractPrecision()
    {
        return Gpu::DtypeCode<U>() == JETGPU_C128 ? JETGPU_PREC_FP32 : Gpu::GetPrecision();
    }

    // Tensor::ContractTensors (reference Tensor.hpp:708-752).
    template <class U = T>
    static Tensor<U> ContractTensors(const Tensor<U> &A, const Tensor<U> &B)
    {
        const ContractionLayout l = LayoutOf<U>(A, B);
        Tensor<U> C(l.c_indices, l.c_shape);
        C.AllocateDevice();
        const int dt = Gpu::DtypeCode<U>();
        const int prec = ContractPrecision<U>();
        const size_t ws = jetgpu_contract_workspace_size(
            (int)l.a_shape.size(), l.a_shape.data(), l.a_perm.data(), (int)l.b_shape.size(),
            l.b_shape.data(), l.b_perm.data(), l.m, l.n, l.k, dt, prec);
        Gpu::DeviceBuffer work(ws);
        Gpu::Check(jetgpu_contract(A.GetDeviceData(), (int)l.a_shape.size(), l.a_shape.data(),
                                   l.a_perm.data(), B.GetDeviceData(), (int)l.b_shape.size(),
                                   l.b_shape.data(), l.b_perm.data(), C.dev_.get(), l.m, l.n, l.k,
                                   dt, prec, JETGPU_ALGO_4M, 0, 0, work.get(), work.size(),
                                   Gpu::Stream()),
                   "ContractTensors");
        C.MarkDeviceWritten();
        return C;
    }
    Tensor<T> ContractWithTensor(const Tensor<T> &other) const
    {
        return ContractTensors<T>(*this, other);
    }

    // Permuter front-end checks (reference permute/Permuter.hpp:99-117).
    static void ValidateOrdering(const std::vector<std::string> &current,
                                 const std::vector<std::string> &target)
    {
        std::vector<std::string> a = current, b = target;
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        JET_ABORT_IF(std::adjacent_find(a.begin(), a.end()) != a.end(),
                     "Duplicate existing indices found. Please ensure indices are unique.");
        JET_ABORT_IF(std::adjacent_find(b.begin(), b.end()) != b.end(),
                     "Duplicate transpose indices found. Please ensure indices are unique.");
        JET_ABORT_IF_NOT(a == b,
                         "New indices are an invalid permutation of the existing indices");
    }

  private:
    std::vector<std::string> indices_;
    std::vector<size_t> shape_;
    mutable std::unordered_map<std::string, size_t> index_to_dimension_;
    mutable bool dims_built_ = false;
    size_t size_ = 1;
    // Host mirror and device copy; an invalid pair means "all zeros".
    mutable std::vector<T> host_;
    mutable bool host_valid_ = false;
    mutable Gpu::DeviceBuffer dev_;
    mutable bool dev_valid_ = false;
    mutable std::mutex sync_;

    template <class> friend class Tensor;

    static int32_t PositionOf(const std::vector<std::string> &v, const std::string &x)
    {
        return static_cast<int32_t>(std::find(v.begin(), v.end(), x) - v.begin());
    }

    bool IsZeroSentinel() const
    {
        return indices_.empty() && shape_.empty() && size_ == 1 && HostView()[0] == T{0};
    }

    void AllocateDevice() const
    {
        if (dev_.get() == nullptr || dev_.size() < size_ * sizeof(T))
            dev_ = Gpu::DeviceBuffer(size_ * sizeof(T));
    }

    void MarkDeviceWritten()
    {
        dev_valid_ = true;
        host_valid_ = false;
    }

    void SyncDevice() const
    {
        std::lock_guard<std::mutex> lock(sync_);
        if (dev_valid_)
            return;
        AllocateDevice();
        if (host_valid_)
            Gpu::Check(jetgpu_memcpy(dev_.get(), host_.data(), size_ * sizeof(T), 0,
                                     Gpu::Stream()),
                       "upload");
        else
            Gpu::Check(jetgpu_memset_zero(dev_.get(), size_ * sizeof(T), Gpu::Stream()),
                       "zero fill");
        dev_valid_ = true;
    }

    const std::vector<T> &HostView() const
    {
        std::lock_guard<std::mutex> lock(sync_);
        if (!host_valid_) {
            host_.assign(size_, T{0});
            if (dev_valid_) {
                Gpu::Check(jetgpu_memcpy(host_.data(), dev_.get(), size_ * sizeof(T), 1,
                                         Gpu::Stream()),
                           "download");
                Gpu::Synchronize();
            }
            host_valid_ = true;
        }
        return host_;
    }

    std::vector<T> &HostMutable()
    {
        HostView();
        dev_valid_ = false;
        return host_;
    }

    void CopyDataFrom(const Tensor &other)
    {
        size_ = other.size_;
        if (other.dev_valid_) {
            AllocateDevice();
            Gpu::Check(jetgpu_memcpy(dev_.get(), other.dev_.get(), size_ * sizeof(T), 2,
                                     Gpu::Stream()),
                       "device copy");
            dev_valid_ = true;
            host_valid_ = false;
        }
        else {
            host_ = other.host_;
            host_valid_ = other.host_valid_;
            dev_valid_ = false;
        }
    }

    void CopyFrom(const Tensor &other)
    {
        InitIndicesAndShape(other.indices_, other.shape_);
        CopyDataFrom(other);
    }

    void MoveFrom(Tensor &&other) noexcept
    {
        indices_ = std::move(other.indices_);
        shape_ = std::move(other.shape_);
        index_to_dimension_ = std::move(other.index_to_dimension_);
        dims_built_ = other.dims_built_;
        other.index_to_dimension_.clear();
        other.dims_built_ = false;
        size_ = other.size_;
        host_ = std::move(other.host_);
        host_valid_ = other.host_valid_;
        dev_ = std::move(other.dev_);
        dev_valid_ = other.dev_valid_;
        other.host_valid_ = false;
        other.dev_valid_ = false;
    }
};

template <class T> inline std::ostream &operator<<(std::ostream &out, const Tensor<T> &t)
{
    out << "Size = " << t.GetSize() << std::endl << "Indices = {";
    for (size_t i = 0; i < t.GetIndices().size(); ++i)
        out << (i ? "  " : "") << t.GetIndices()[i];
    out << "}" << std::endl << "Data = {";
    const auto &d = t.GetData();
    for (size_t i = 0; i < d.size(); ++i)
        out << (i ? "  " : "") << d[i];
    out << "}";
    return out;
}

} // namespace Jet
