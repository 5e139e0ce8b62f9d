// Jet::CudaTensor checks (reference behaviour: test/Test_CudaTensor.cpp).
// Built and run by tests/test_cuda_tensor.py; prints one line per failed
// check and "ALL OK" when every check holds. Column-major semantics: a
// CudaTensor's data vary fastest along its first index.
#include <cmath>
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "Jet.hpp"

using namespace Jet;
using c64_dev = cuComplex;
using c128_dev = cuDoubleComplex;
using c64_host = std::complex<float>;
using c128_host = std::complex<double>;

static int failures = 0;
#define CHECK(...)                                                                     \
    do {                                                                               \
        if (!(__VA_ARGS__)) {                                                          \
            ++failures;                                                                \
            std::printf("FAILED line %d: %s\n", __LINE__, #__VA_ARGS__);              \
        }                                                                              \
    } while (0)

template <class F> static std::string ThrowsWith(F f)
{
    try {
        f();
    }
    catch (const Jet::Exception &e) {
        return e.what();
    }
    return "";
}

static bool Contains(const std::string &s, const std::string &sub)
{
    return s.find(sub) != std::string::npos;
}

static std::vector<c64_dev> Dev(const std::vector<c64_host> &h)
{
    std::vector<c64_dev> d(h.size());
    for (size_t i = 0; i < h.size(); ++i)
        d[i] = make_cuComplex(h[i].real(), h[i].imag());
    return d;
}

static void Construction()
{
    CudaTensor<> t;
    CHECK(t.GetIndices().empty());
    CHECK(t.GetShape().empty());
    CHECK(t.GetSize() == 1);
    CHECK(t.GetHostDataVector() == std::vector<c64_host>{{0, 0}});

    CudaTensor<> s({2, 3});
    CHECK((s.GetIndices() == std::vector<std::string>{"?a", "?b"}));
    CHECK(s.GetSize() == 6);
    CHECK(s.GetIndexToDimension().at("?b") == 3);

    const std::vector<c64_host> v{{1, 2}, {3, 4}, {5, 6}, {7, 8}};
    CudaTensor<> d({"i", "j"}, {2, 2}, Dev(v));
    CHECK(d.GetHostDataVector() == v);
    CudaTensor<> copy(d);
    CHECK(copy.GetHostDataVector() == v);
    CHECK(copy.GetIndices() == d.GetIndices());
    CudaTensor<> assigned;
    assigned = d;
    CHECK(assigned.GetHostDataVector() == v);

    // From / to Jet::Tensor: labels and shape reversed, data unchanged.
    Tensor<c64_host> host({"i", "j"}, {2, 2}, v);
    CudaTensor<> from_host(host);
    CHECK((from_host.GetIndices() == std::vector<std::string>{"j", "i"}));
    CHECK(from_host.GetHostDataVector() == v);
    CudaTensor<> vec({"i"}, {2}, Dev({{2, 0}, {0, 1}}));
    CHECK(static_cast<Tensor<c64_host>>(vec) ==
          Tensor<c64_host>({"i"}, {2}, {{2, 0}, {0, 1}}));
}

static void RenameReshapeSlice()
{
    CudaTensor<> t({"a", "b"}, {3, 2});
    t.RenameIndex(1, "z");
    CHECK((t.GetIndices() == std::vector<std::string>{"a", "z"}));
    CHECK(t.GetIndexToDimension().at("z") == 2);
    t.RenameIndex(0, "a");
    CHECK(t.GetIndexToDimension().at("a") == 3);
    CHECK(Contains(ThrowsWith([&] { t.RenameIndex(1, "a"); }),
                   "Renaming index to already existing value is not allowed."));

    const std::vector<c64_host> six{{1, 0}, {2, 0}, {3, 0}, {4, 0}, {5, 0}, {6, 0}};
    CudaTensor<> m({"x", "y"}, {2, 3}, Dev(six));
    auto r = m.Reshape({3, 2});
    CHECK((r.GetShape() == std::vector<size_t>{3, 2}));
    CHECK((r.GetIndices() == std::vector<std::string>{"?a", "?b"}));
    CHECK(r.GetHostDataVector() == six);
    CHECK(Contains(ThrowsWith([&] { CudaTensor<>::Reshape(m, {3, 3}); }),
                   "Size is inconsistent between tensors."));

    // Column-major: m(x, y) = six[x + 2 y].
    CHECK((m.SliceIndex("x", 0).GetHostDataVector() == std::vector<c64_host>{{1, 0}, {3, 0}, {5, 0}}));
    CHECK((m.SliceIndex("x", 1).GetHostDataVector() == std::vector<c64_host>{{2, 0}, {4, 0}, {6, 0}}));
    CHECK((m.SliceIndex("y", 0).GetHostDataVector() == std::vector<c64_host>{{1, 0}, {2, 0}}));
    CHECK((m.SliceIndex("y", 2).GetHostDataVector() == std::vector<c64_host>{{5, 0}, {6, 0}}));
    CHECK((m.SliceIndex("y", 1).GetIndices() == std::vector<std::string>{"x"}));

    // Transpose: mt(y, x) = m(x, y), column-major over (y, x).
    auto mt = m.Transpose(std::vector<std::string>{"y", "x"});
    CHECK((mt.GetShape() == std::vector<size_t>{3, 2}));
    CHECK((mt.GetHostDataVector() ==
           std::vector<c64_host>{{1, 0}, {3, 0}, {5, 0}, {2, 0}, {4, 0}, {6, 0}}));
    CHECK(mt.Transpose(std::vector<size_t>{1, 0}).GetHostDataVector() == six);
    CHECK(Contains(ThrowsWith([&] { m.Transpose(std::vector<size_t>{0}); }),
                   "Size of ordering must match number of tensor indices."));
}

static void Contractions()
{
    CudaTensor<> t0({"a", "b"}, {2, 2}, Dev({{0, 0}, {1, 0}, {1, 0}, {0, 0}}));
    CudaTensor<> t1({"b"}, {2}, Dev({{1, 0}, {0, 0}}));
    auto t2 = CudaTensor<>::ContractTensors<c64_dev>(t0, t1);
    CHECK(static_cast<Tensor<c64_host>>(t2) == Tensor<c64_host>({"a"}, {2}, {{0, 0}, {1, 0}}));

    std::vector<c64_dev> q1(24, make_cuComplex(0.5f, 0.25f)), q2(24, make_cuComplex(0.5f, 0.25f));
    CudaTensor<> a({"a", "b", "c"}, {2, 3, 4}, q1);
    CudaTensor<> b({"b", "c", "d"}, {3, 4, 2}, q2);
    auto c = a.ContractTensors(b);
    CHECK((c.GetIndices() == std::vector<std::string>{"a", "d"}));
    CHECK(c.GetHostDataVector() == std::vector<c64_host>(4, c64_host(2.25f, 3.0f)));

    CudaTensor<> s1({"a", "b"}, {2, 2}, std::vector<c64_dev>(4, make_cuComplex(1, 0)));
    CudaTensor<> s2({"a", "b"}, {2, 2}, std::vector<c64_dev>(4, make_cuComplex(1, 0)));
    auto sc = CudaTensor<>::ContractTensors<c64_dev>(s1, s2);
    CHECK(static_cast<Tensor<c64_host>>(sc) == Tensor<c64_host>({}, {}, {{4, 0}}));

    // Random tensors against Jet::Tensor (row-major, reversed labels).
    CudaTensor<> r1({"a", "b", "c"}, {2, 3, 5});
    CudaTensor<> r2({"c", "b", "d"}, {5, 3, 4});
    r1.FillRandom(7);
    r2.FillRandom(7);
    Tensor<c64_host> h1(r1), h2(r2);
    CHECK((h1.GetIndices() == std::vector<std::string>{"c", "b", "a"}));
    auto h3 = Tensor<c64_host>::ContractTensors(h1, h2);
    auto r3 = r1.ContractTensors(r2);
    Tensor<c64_host> h3c(r3);
    CHECK(h3c.GetIndices() == CudaTensorHelpers::ReverseVector(h3.GetIndices()));
    // h3 is row-major over (c-free labels of h1 ++ h2) = (a, d) order reversed.
    const auto &d1 = h3c.GetData();
    const auto &d2 = h3.GetData();
    bool close = d1.size() == 8;
    for (size_t i = 0; close && i < 8; ++i) {
        const size_t row = i % 2, col = i / 2; // r3(a, d) column-major
        const auto want = d2[row * 4 + col];   // h3(a, d) row-major
        close = std::abs(d1[i] - want) <= 1e-5f * std::abs(want) + 1e-6f;
    }
    CHECK(close);
    r1.FillRandom(7);
    CudaTensor<> r1b({"a", "b", "c"}, {2, 3, 5});
    r1b.FillRandom(7);
    CHECK(r1.GetHostDataVector() == r1b.GetHostDataVector());
    r1b.FillRandom(8);
    CHECK(r1.GetHostDataVector() != r1b.GetHostDataVector());

    // Plan + preallocated output, with C in the contraction's order and in
    // the reversed order.
    CudaTensor<> out({"a", "d"}, {2, 4});
    CudaTensor<>::CudaContractionPlan plan;
    CudaTensor<>::GetCudaContractionPlan<c64_dev>(plan, r1, r2, out);
    CudaTensor<>::ContractTensorsWithoutAllocation<c64_dev>(r1, r2, out, plan);
    CHECK(out.GetHostDataVector() == r3.GetHostDataVector());
    CudaTensor<> out_t({"d", "a"}, {4, 2});
    CudaTensor<>::CudaContractionPlan plan_t;
    CudaTensor<>::GetCudaContractionPlan<c64_dev>(plan_t, r1, r2, out_t);
    CudaTensor<>::ContractTensorsWithoutAllocation<c64_dev>(r1, r2, out_t, plan_t);
    CHECK(out_t.GetHostDataVector() ==
          r3.Transpose(std::vector<std::string>{"d", "a"}).GetHostDataVector());

    // complex128.
    std::vector<c128_dev> z(24, make_cuDoubleComplex(0.5, 0.25));
    CudaTensor<c128_dev> za({"a", "b", "c"}, {2, 3, 4}, z);
    CudaTensor<c128_dev> zb({"b", "c", "d"}, {3, 4, 2}, z);
    CHECK(za.ContractTensors(zb).GetHostDataVector() ==
          std::vector<c128_host>(4, c128_host(2.25, 3.0)));
}

static void Additions()
{
    CudaTensor<> l0({}, {}, Dev({{1, 0}}));
    CudaTensor<> r0({}, {}, Dev({{2, 4}}));
    CHECK(CudaTensor<>::AddTensors(l0, r0).GetHostDataVector() == std::vector<c64_host>{{3, 4}});

    CudaTensor<> lv({"i"}, {3}, Dev({{1, 0}, {0, 2}, {3, 0}}));
    CudaTensor<> rv({"i"}, {3}, Dev({{1, 0}, {0, 2}, {0, 3}}));
    CHECK((lv.AddTensor(rv).GetHostDataVector() == std::vector<c64_host>{{2, 0}, {0, 4}, {3, 3}}));

    CudaTensor<> lm({"i", "j"}, {2, 2}, Dev({{1, 0}, {2, 0}, {3, 0}, {4, 0}}));
    CudaTensor<> rm({"j", "i"}, {2, 2}, Dev({{0, 1}, {0, 2}, {0, 3}, {0, 4}}));
    CHECK((CudaTensor<>::AddTensors(lm, rm).GetHostDataVector() ==
           std::vector<c64_host>{{1, 1}, {2, 3}, {3, 2}, {4, 4}}));
    CudaTensor<> zero;
    CHECK(CudaTensor<>::AddTensors(zero, lm).GetHostDataVector() == lm.GetHostDataVector());
    CudaTensor<> other({"k"}, {2});
    CHECK(Contains(ThrowsWith([&] { CudaTensor<>::AddTensors(lm, other); }),
                   "Tensor addition with disjoint indices is not supported."));
}

static void NetworkWithCudaTensors()
{
    // A ring of four 2x2 tensors contracted by TaskBasedContractor over
    // CudaTensor, against the same network over Jet::Tensor.
    TensorNetwork<CudaTensor<>> tn;
    TensorNetwork<Tensor<c64_host>> tn_host;
    const std::vector<std::vector<std::string>> labels{{"i", "j"}, {"j", "k"}, {"k", "l"}, {"l", "i"}};
    for (size_t t = 0; t < labels.size(); ++t) {
        CudaTensor<> ct(labels[t], {2, 2});
        ct.FillRandom(100 + t);
        Tensor<c64_host> ht(ct); // reversed labels, same data
        tn.AddTensor(ct, {});
        tn_host.AddTensor(ht, {});
    }
    const PathInfo::Path path{{0, 1}, {2, 3}, {4, 5}};
    PathInfo info(tn, path);
    TaskBasedContractor<CudaTensor<>> tbc;
    tbc.AddContractionTasks(tn, info);
    tbc.Contract().wait();
    const auto got = tbc.GetResults()[0].GetHostDataVector();
    const auto want = tn_host.Contract(path).GetData();
    CHECK(got.size() == 1 && want.size() == 1 &&
          std::abs(got[0] - want[0]) <= 1e-5f * std::abs(want[0]));
}

int main()
{
    try {
        Construction();
        RenameReshapeSlice();
        Contractions();
        Additions();
        NetworkWithCudaTensors();
    }
    catch (const std::exception &e) {
        std::printf("FAILED with exception: %s\n", e.what());
        return 2;
    }
    if (failures) {
        std::printf("%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
