// Device memory exhaustion injected on the host: with the library pool capped
// (jetgpu_set_pool_limit), a contraction's uploads or workspace fail before
// any CUDA call and the C++ API raises Jet::Exception; lifting the cap makes
// the same contraction succeed with the result of an uncapped run, and no
// device bytes stay held by the failed attempts. Covers Tensor::ContractTensors,
// TaskBasedContractor (the exception reaches the caller through the future)
// and SlicedContractor. Built and run by tests/test_cpp_api.py; prints
// "ALL OK" when every check holds.
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "Jet.hpp"

using namespace Jet;
using c64 = std::complex<float>;

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

static Tensor<c64> Random(const std::vector<std::string> &labels, const std::vector<size_t> &dims,
                          size_t seed)
{
    Tensor<c64> t(labels, dims);
    t.FillRandom(seed);
    return t;
}

// A fresh host-only copy: its device copy is made by the next contraction.
static Tensor<c64> HostCopy(const Tensor<c64> &t)
{
    return Tensor<c64>(t.GetIndices(), t.GetShape(), t.GetData());
}

static void PairwiseContraction()
{
    const auto a = Random({"i", "j"}, {128, 64}, 1);
    const auto b = Random({"j", "k"}, {64, 96}, 2);
    const auto want = Tensor<c64>::ContractTensors(HostCopy(a), HostCopy(b)).GetData();

    const size_t base = jetgpu_pool_bytes_in_use();
    {
        const auto a2 = HostCopy(a), b2 = HostCopy(b);
        jetgpu_set_pool_limit(base + 4096);
        const auto msg = ThrowsWith([&] { Tensor<c64>::ContractTensors(a2, b2); });
        CHECK(Contains(msg, "device memory limit"));
        jetgpu_set_pool_limit(0);
        const auto got = Tensor<c64>::ContractTensors(a2, b2).GetData();
        CHECK(got == want);
    }
    CHECK(jetgpu_pool_bytes_in_use() == base);
}

static TensorNetwork<Tensor<c64>> Ring(size_t seed)
{
    TensorNetwork<Tensor<c64>> tn;
    const std::vector<std::vector<std::string>> labels{{"a", "b"}, {"b", "c"}, {"c", "d"},
                                                       {"d", "a"}};
    for (size_t t = 0; t < labels.size(); ++t)
        tn.AddTensor(Random(labels[t], {32, 32}, seed + t), {});
    return tn;
}

static void TaskBasedNetwork()
{
    const PathInfo::Path path{{0, 1}, {2, 3}, {4, 5}};
    c64 want;
    {
        auto tn = Ring(10);
        PathInfo info(tn, path);
        TaskBasedContractor<Tensor<c64>> tbc;
        tbc.AddContractionTasks(tn, info);
        tbc.Contract().get();
        want = tbc.GetResults()[0].GetData()[0];
    }
    const size_t base = jetgpu_pool_bytes_in_use();
    {
        auto tn = Ring(10);
        PathInfo info(tn, path);
        TaskBasedContractor<Tensor<c64>> tbc;
        tbc.AddContractionTasks(tn, info);
        jetgpu_set_pool_limit(base + 4096);
        const auto msg = ThrowsWith([&] { tbc.Contract().get(); });
        jetgpu_set_pool_limit(0);
        CHECK(Contains(msg, "device memory limit"));
    }
    CHECK(jetgpu_pool_bytes_in_use() == base);
    {
        auto tn = Ring(10);
        PathInfo info(tn, path);
        TaskBasedContractor<Tensor<c64>> tbc;
        tbc.AddContractionTasks(tn, info);
        tbc.Contract().get();
        CHECK(tbc.GetResults()[0].GetData()[0] == want);
    }
}

static void SlicedNetwork()
{
    const PathInfo::Path path{{0, 1}, {2, 3}, {4, 5}};
    std::vector<std::complex<double>> want;
    {
        auto tn = Ring(20);
        SlicedContractor<c64> sc(tn, path, {"a"});
        sc.SetBatchSize(8);
        want = sc.Contract();
    }
    const size_t base = jetgpu_pool_bytes_in_use();
    {
        auto tn = Ring(20);
        SlicedContractor<c64> sc(tn, path, {"a"});
        sc.SetBatchSize(8);
        jetgpu_set_pool_limit(base + 4096);
        const auto msg = ThrowsWith([&] { sc.Contract(); });
        jetgpu_set_pool_limit(0);
        CHECK(Contains(msg, "device memory limit"));
        // The same contractor plans again once memory is available.
        CHECK(sc.Contract() == want);
    }
    CHECK(jetgpu_pool_bytes_in_use() == base);
}

int main()
{
    try {
        PairwiseContraction();
        TaskBasedNetwork();
        SlicedNetwork();
    }
    catch (const std::exception &e) {
        jetgpu_set_pool_limit(0);
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
