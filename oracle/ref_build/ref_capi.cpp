// C entry points over the UNMODIFIED reference Jet headers, compiled from the
// reference tree by oracle/ref_build/Makefile into oracle/_ref/libjetref.so.
//
// TEST INFRASTRUCTURE ONLY. This library is the CPU reference that pins the
// oracle restatement (oracle/jet_oracle.py, oracle/jet_oracle.c) and generates
// golden fixtures under tests/golden/. Nothing in jet_gb300/ links or loads it.
//
// Reference entry points wrapped here:
//   Jet::Tensor<T>::Transpose          include/jet/Tensor.hpp:578-642
//   Jet::Permuter<QFlex|Default>       include/jet/permute/Permuter.hpp:49-119
//   Jet::Tensor<T>::ContractTensors    include/jet/Tensor.hpp:708-752
//   Jet::Tensor<T>::SliceIndex         include/jet/Tensor.hpp:493-526
//   Jet::Tensor<T>::AddTensors         include/jet/Tensor.hpp:412-454
//   Jet::TensorNetwork::{SliceIndices,Contract}  include/jet/TensorNetwork.hpp:210-328
//   Jet::PathInfo totals               include/jet/PathInfo.hpp:157-239
//
// Labels cross this boundary as one comma-separated string ("a,b,c"); data as
// interleaved (re, im) arrays of float (dtype 0) or double (dtype 1).
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "jet/PathInfo.hpp"
#include "jet/Tensor.hpp"
#include "jet/TensorNetwork.hpp"

namespace {

thread_local std::string g_err;

std::vector<std::string> SplitLabels(const char *s)
{
    std::vector<std::string> out;
    if (s == nullptr || *s == '\0')
        return out;
    std::string cur;
    for (const char *p = s; *p; ++p) {
        if (*p == ',') {
            out.push_back(cur);
            cur.clear();
        }
        else {
            cur.push_back(*p);
        }
    }
    out.push_back(cur);
    return out;
}

std::string JoinLabels(const std::vector<std::string> &v)
{
    std::string s;
    for (size_t i = 0; i < v.size(); ++i) {
        if (i)
            s += ",";
        s += v[i];
    }
    return s;
}

template <class T>
Jet::Tensor<T> MakeTensor(size_t rank, const size_t *shape, const char *labels,
                          const void *data)
{
    std::vector<size_t> sh(shape, shape + rank);
    std::vector<std::string> lb = SplitLabels(labels);
    size_t n = Jet::Utilities::ShapeToSize(sh);
    std::vector<T> d(n);
    std::memcpy(d.data(), data, n * sizeof(T));
    return Jet::Tensor<T>(lb, sh, d);
}

template <class T>
int ExportTensor(const Jet::Tensor<T> &t, size_t *rank_out, size_t *shape_out,
                 char *labels_out, size_t labels_cap, void *data_out,
                 size_t data_cap)
{
    const auto &sh = t.GetShape();
    const auto &lb = t.GetIndices();
    *rank_out = lb.size();
    for (size_t i = 0; i < sh.size(); ++i)
        shape_out[i] = sh[i];
    std::string joined = JoinLabels(lb);
    if (joined.size() + 1 > labels_cap) {
        g_err = "label buffer too small";
        return 1;
    }
    std::memcpy(labels_out, joined.c_str(), joined.size() + 1);
    if (t.GetSize() > data_cap) {
        g_err = "data buffer too small";
        return 1;
    }
    std::memcpy(data_out, t.GetData().data(), t.GetSize() * sizeof(T));
    return 0;
}

template <class T>
int Contract(size_t ra, const size_t *sa, const char *la, const void *a,
             size_t rb, const size_t *sb, const char *lb, const void *b,
             size_t *rc, size_t *sc, char *lc, size_t lc_cap, void *c,
             size_t c_cap)
{
    auto A = MakeTensor<T>(ra, sa, la, a);
    auto B = MakeTensor<T>(rb, sb, lb, b);
    auto C = Jet::Tensor<T>::ContractTensors(A, B);
    return ExportTensor(C, rc, sc, lc, lc_cap, c, c_cap);
}

template <class T, class Backend>
int PermuterTranspose(size_t rank, const size_t *shape, const char *old_labels,
                      const char *new_labels, const void *in, size_t n, void *out)
{
    std::vector<size_t> sh(shape, shape + rank);
    std::vector<T> d(n);
    if (n)
        std::memcpy(d.data(), in, n * sizeof(T));
    Jet::Permuter<Backend> permuter;
    auto r = permuter.Transpose(d, sh, SplitLabels(old_labels),
                                SplitLabels(new_labels));
    std::memcpy(out, r.data(), r.size() * sizeof(T));
    return 0;
}

template <class T>
int NetworkContract(size_t ntensors, const size_t *ranks,
                    const size_t *shapes_flat, const char *const *labels,
                    const void *const *datas, size_t npath,
                    const size_t *path_pairs, const char *sliced_labels,
                    unsigned long long slice_value, double *flops_out,
                    double *memory_out, size_t *rc, size_t *sc, char *lc,
                    size_t lc_cap, void *c, size_t c_cap)
{
    Jet::TensorNetwork<Jet::Tensor<T>> tn;
    size_t off = 0;
    for (size_t i = 0; i < ntensors; ++i) {
        tn.AddTensor(MakeTensor<T>(ranks[i], shapes_flat + off, labels[i],
                                   datas[i]),
                     {});
        off += ranks[i];
    }
    auto sliced = SplitLabels(sliced_labels);
    if (!sliced.empty())
        tn.SliceIndices(sliced, slice_value);
    std::vector<std::pair<size_t, size_t>> path(npath);
    for (size_t i = 0; i < npath; ++i)
        path[i] = {path_pairs[2 * i], path_pairs[2 * i + 1]};
    Jet::PathInfo info(tn, path);
    if (flops_out)
        *flops_out = info.GetTotalFlops();
    if (memory_out)
        *memory_out = info.GetTotalMemory();
    const auto &res = tn.Contract(path);
    return ExportTensor(res, rc, sc, lc, lc_cap, c, c_cap);
}

} // namespace

extern "C" {

const char *jetref_last_error(void) { return g_err.c_str(); }

// Tensor::Transpose (QFlex<1024,32> for power-of-2 sizes with Default<1024>
// fallback, exactly as Tensor.hpp:594-611 selects).
int jetref_tensor_transpose(int dtype, size_t rank, const size_t *shape,
                            const char *old_labels, const char *new_labels,
                            const void *in, void *out)
{
    try {
        if (dtype == 0) {
            auto A = MakeTensor<std::complex<float>>(rank, shape, old_labels, in);
            auto R = Jet::Tensor<std::complex<float>>::Transpose(
                A, SplitLabels(new_labels));
            std::memcpy(out, R.GetData().data(), R.GetSize() * 8);
        }
        else {
            auto A = MakeTensor<std::complex<double>>(rank, shape, old_labels, in);
            auto R = Jet::Tensor<std::complex<double>>::Transpose(
                A, SplitLabels(new_labels));
            std::memcpy(out, R.GetData().data(), R.GetSize() * 16);
        }
        return 0;
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

// Permuter<Backend>::Transpose of n_data elements, backend 0 = DefaultPermuter<1024>,
// 1 = QFlexPermuter<1024,32>, 2 = QFlexPermuter<64,32> (the reference test's
// "insufficient BLOCKSIZE" configuration), 3 = <128,64>, 4 = <256,2>,
// 5 = <64,2>, 6 = <2048,1024>, 7 = <512,32>. complex<float> only.
int jetref_permuter_transpose(int backend, size_t rank, const size_t *shape,
                              const char *old_labels, const char *new_labels,
                              const void *in, size_t n_data, void *out)
{
    using T = std::complex<float>;
    try {
        if (backend == 0)
            return PermuterTranspose<T, Jet::DefaultPermuter<1024>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 1)
            return PermuterTranspose<T, Jet::QFlexPermuter<1024, 32>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 2)
            return PermuterTranspose<T, Jet::QFlexPermuter<64, 32>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 3)
            return PermuterTranspose<T, Jet::QFlexPermuter<128, 64>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 4)
            return PermuterTranspose<T, Jet::QFlexPermuter<256, 2>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 5)
            return PermuterTranspose<T, Jet::QFlexPermuter<64, 2>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        if (backend == 6)
            return PermuterTranspose<T, Jet::QFlexPermuter<2048, 1024>>(
                rank, shape, old_labels, new_labels, in, n_data, out);
        return PermuterTranspose<T, Jet::QFlexPermuter<512, 32>>(
            rank, shape, old_labels, new_labels, in, n_data, out);
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

int jetref_contract(int dtype, size_t ra, const size_t *sa, const char *la,
                    const void *a, size_t rb, const size_t *sb, const char *lb,
                    const void *b, size_t *rc, size_t *sc, char *lc,
                    size_t lc_cap, void *c, size_t c_cap)
{
    try {
        if (dtype == 0)
            return Contract<std::complex<float>>(ra, sa, la, a, rb, sb, lb, b,
                                                 rc, sc, lc, lc_cap, c, c_cap);
        return Contract<std::complex<double>>(ra, sa, la, a, rb, sb, lb, b, rc,
                                              sc, lc, lc_cap, c, c_cap);
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

int jetref_slice_index(int dtype, size_t rank, const size_t *shape,
                       const char *labels, const void *in, const char *index,
                       size_t value, size_t *rc, size_t *sc, char *lc,
                       size_t lc_cap, void *c, size_t c_cap)
{
    try {
        if (dtype == 0) {
            auto A = MakeTensor<std::complex<float>>(rank, shape, labels, in);
            auto R = Jet::Tensor<std::complex<float>>::SliceIndex(A, index, value);
            return ExportTensor(R, rc, sc, lc, lc_cap, c, c_cap);
        }
        auto A = MakeTensor<std::complex<double>>(rank, shape, labels, in);
        auto R = Jet::Tensor<std::complex<double>>::SliceIndex(A, index, value);
        return ExportTensor(R, rc, sc, lc, lc_cap, c, c_cap);
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

int jetref_add_tensors(int dtype, size_t ra, const size_t *sa, const char *la,
                       const void *a, size_t rb, const size_t *sb,
                       const char *lb, const void *b, size_t *rc, size_t *sc,
                       char *lc, size_t lc_cap, void *c, size_t c_cap)
{
    try {
        if (dtype == 0) {
            auto A = MakeTensor<std::complex<float>>(ra, sa, la, a);
            auto B = MakeTensor<std::complex<float>>(rb, sb, lb, b);
            auto C = Jet::Tensor<std::complex<float>>::AddTensors(A, B);
            return ExportTensor(C, rc, sc, lc, lc_cap, c, c_cap);
        }
        auto A = MakeTensor<std::complex<double>>(ra, sa, la, a);
        auto B = MakeTensor<std::complex<double>>(rb, sb, lb, b);
        auto C = Jet::Tensor<std::complex<double>>::AddTensors(A, B);
        return ExportTensor(C, rc, sc, lc, lc_cap, c, c_cap);
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

// Builds a TensorNetwork from `ntensors` leaves, optionally slices
// `sliced_labels` at `slice_value` (TensorNetwork::SliceIndices), runs
// TensorNetwork::Contract(path) and returns the last node's tensor plus the
// PathInfo flop and memory totals of the (sliced) network.
int jetref_network_contract(int dtype, size_t ntensors, const size_t *ranks,
                            const size_t *shapes_flat,
                            const char *const *labels,
                            const void *const *datas, size_t npath,
                            const size_t *path_pairs, const char *sliced_labels,
                            unsigned long long slice_value, double *flops_out,
                            double *memory_out, size_t *rc, size_t *sc,
                            char *lc, size_t lc_cap, void *c, size_t c_cap)
{
    try {
        if (dtype == 0)
            return NetworkContract<std::complex<float>>(
                ntensors, ranks, shapes_flat, labels, datas, npath, path_pairs,
                sliced_labels, slice_value, flops_out, memory_out, rc, sc, lc,
                lc_cap, c, c_cap);
        return NetworkContract<std::complex<double>>(
            ntensors, ranks, shapes_flat, labels, datas, npath, path_pairs,
            sliced_labels, slice_value, flops_out, memory_out, rc, sc, lc,
            lc_cap, c, c_cap);
    }
    catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}

} // extern "C"
