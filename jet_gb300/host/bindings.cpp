// Python bindings of the GB300 Jet host API (module jet_gb300._jet_bindings).
//
// Mirrors the Python surface of the reference's jet.bindings module
// (python/src/*.hpp): classes TensorC64/TensorC128, TensorNetworkC64/C128,
// PathInfo, TaskBasedContractorC64/C128 and the free functions
// contract_tensors, add_tensors, conj, reshape, slice_index, transpose. The
// tensors behind these classes live in GPU memory (jet/Tensor.hpp).
#include <pybind11/complex.h>
#include <pybind11/operators.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <sstream>

#include "Jet.hpp"

namespace py = pybind11;

namespace {

template <class T> std::string Suffix()
{
    return std::is_same_v<T, std::complex<float>> ? "C64" : "C128";
}

template <class T> void BindTensor(py::module_ &m)
{
    using tensor_t = Jet::Tensor<T>;
    const std::string name = "Tensor" + Suffix<T>();
    py::class_<tensor_t>(m, name.c_str(), "Labelled complex tensor stored on the GPU.")
        .def(py::init<>())
        .def(py::init<const std::vector<size_t> &>(), py::arg("shape"))
        .def(py::init<const std::vector<std::string> &, const std::vector<size_t> &>(),
             py::arg("indices"), py::arg("shape"))
        .def(py::init<const std::vector<std::string> &, const std::vector<size_t> &,
                      const std::vector<T> &>(),
             py::arg("indices"), py::arg("shape"), py::arg("data"))
        .def(py::init<const tensor_t &>(), py::arg("other"))
        .def_property_readonly_static("dtype",
                                      [](py::object) {
                                          return std::is_same_v<T, std::complex<float>>
                                                     ? "complex64"
                                                     : "complex128";
                                      })
        .def_property(
            "data", [](const tensor_t &t) { return t.GetData(); },
            [](tensor_t &t, const std::vector<T> &d) { t.SetData(d); })
        .def_property("shape", &tensor_t::GetShape, &tensor_t::SetShape)
        .def_property_readonly("indices", &tensor_t::GetIndices)
        .def_property_readonly("index_to_dimension_map", &tensor_t::GetIndexToDimension)
        .def_property_readonly("scalar", [](const tensor_t &t) { return t.GetScalar(); })
        .def_property_readonly("size", &tensor_t::GetSize)
        .def("__getitem__", [](const tensor_t &t, size_t pos) { return t[pos]; },
             py::arg("pos"))
        .def("__len__", &tensor_t::GetSize)
        .def("__repr__",
             [](const tensor_t &t) {
                 std::stringstream s;
                 s << t;
                 return s.str();
             })
        .def(py::self == py::self, py::arg("other"))
        .def(py::self != py::self, py::arg("other"))
        .def("fill_random", [](tensor_t &t) { t.FillRandom(); })
        .def("fill_random", [](tensor_t &t, size_t seed) { t.FillRandom(seed); },
             py::arg("seed"))
        .def("init_indices_and_shape", &tensor_t::InitIndicesAndShape, py::arg("indices"),
             py::arg("shape"))
        .def("get_value", &tensor_t::GetValue, py::arg("indices"))
        .def("set_value", &tensor_t::SetValue, py::arg("indices"), py::arg("value"))
        .def("rename_index", &tensor_t::RenameIndex, py::arg("pos"), py::arg("new_label"))
        .def("is_scalar", &tensor_t::IsScalar)
        .def("add_tensor", &tensor_t::AddTensor, py::arg("other"))
        .def("contract_with_tensor", &tensor_t::ContractWithTensor, py::arg("other"))
        .def("slice_index",
             [](const tensor_t &t, const std::string &i, size_t v) { return t.SliceIndex(i, v); },
             py::arg("index"), py::arg("value"))
        .def("reshape", [](const tensor_t &t, const std::vector<size_t> &s) { return t.Reshape(s); },
             py::arg("shape"))
        .def("transpose",
             [](const tensor_t &t, const std::vector<std::string> &l) { return t.Transpose(l); },
             py::arg("indices"))
        .def("transpose",
             [](const tensor_t &t, const std::vector<size_t> &o) { return t.Transpose(o); },
             py::arg("ordering"))
        .def("conj", [](const tensor_t &t) { return t.Conj(); })
        // GPU extras: raw device pointer (for zero-copy interop) and upload.
        .def("device_ptr",
             [](const tensor_t &t) { return reinterpret_cast<uintptr_t>(t.GetDeviceData()); })
        .def("set_device_data",
             [](tensor_t &t, uintptr_t ptr) { t.SetDeviceData(reinterpret_cast<const T *>(ptr)); },
             py::arg("ptr"));

    m.def("conj", [](const tensor_t &t) { return tensor_t::Conj(t); }, py::arg("tensor"));
    // Permuter<Backend>::Transpose on host data (the permuter plugin point):
    // backend "qflex" = QFlexPermuter<>, "qflex64" = QFlexPermuter<64>,
    // "default" = DefaultPermuter<>.
    m.def("permuter_transpose",
          [](const std::vector<T> &data, const std::vector<size_t> &shape,
             const std::vector<std::string> &current, const std::vector<std::string> &target,
             const std::string &backend) {
              if (backend == "qflex")
                  return Jet::Permuter<Jet::QFlexPermuter<>>().Transpose(data, shape, current,
                                                                         target);
              if (backend == "qflex64")
                  return Jet::Permuter<Jet::QFlexPermuter<64>>().Transpose(data, shape, current,
                                                                           target);
              if (backend == "default")
                  return Jet::Permuter<Jet::DefaultPermuter<>>().Transpose(data, shape, current,
                                                                           target);
              throw std::invalid_argument("backend must be qflex, qflex64 or default");
          },
          py::arg("data"), py::arg("shape"), py::arg("current_order"), py::arg("new_order"),
          py::arg("backend") = "qflex");
    // QFlexPermuter<BLOCKSIZE, MIN_DIMS>::CheckPlan: raises the reference's
    // error when its plan rejects the transpose (host only, no device work).
    m.def("qflex_check_plan",
          [](const std::vector<size_t> &shape, const std::vector<std::string> &current,
             const std::vector<std::string> &target, size_t blocksize, size_t min_dims) {
#define JET_QFLEX_CASE(B, M)                                                           \
    if (blocksize == B && min_dims == M)                                               \
        return Jet::QFlexPermuter<B, M>::CheckPlan(shape, current, target);
              JET_QFLEX_CASE(1024, 32)
              JET_QFLEX_CASE(64, 32)
              JET_QFLEX_CASE(128, 64)
              JET_QFLEX_CASE(256, 2)
              JET_QFLEX_CASE(64, 2)
              JET_QFLEX_CASE(2048, 1024)
              JET_QFLEX_CASE(512, 32)
#undef JET_QFLEX_CASE
              throw std::invalid_argument("no QFlexPermuter instantiation for these parameters");
          },
          py::arg("shape"), py::arg("current_order"), py::arg("new_order"), py::arg("blocksize"),
          py::arg("min_dims"));
    m.def("add_tensors", [](const tensor_t &a, const tensor_t &b) { return tensor_t::AddTensors(a, b); },
          py::arg("A"), py::arg("B"));
    m.def("contract_tensors",
          [](const tensor_t &a, const tensor_t &b) { return tensor_t::ContractTensors(a, b); },
          py::arg("A"), py::arg("B"));
    m.def("reshape",
          [](const tensor_t &t, const std::vector<size_t> &s) { return tensor_t::Reshape(t, s); },
          py::arg("tensor"), py::arg("shape"));
    m.def("slice_index",
          [](const tensor_t &t, const std::string &i, size_t v) { return tensor_t::SliceIndex(t, i, v); },
          py::arg("tensor"), py::arg("index"), py::arg("value"));
    m.def("transpose",
          [](const tensor_t &t, const std::vector<std::string> &l) { return tensor_t::Transpose(t, l); },
          py::arg("tensor"), py::arg("new_indices"));
    m.def("transpose",
          [](const tensor_t &t, const std::vector<size_t> &o) { return tensor_t::Transpose(t, o); },
          py::arg("tensor"), py::arg("new_ordering"));
}

template <class T> void BindTensorNetwork(py::module_ &m)
{
    using tensor_t = Jet::Tensor<T>;
    using tn_t = Jet::TensorNetwork<tensor_t>;
    const std::string s = Suffix<T>();
    py::class_<typename tn_t::Node>(m, ("TensorNetworkNode" + s).c_str())
        .def_readonly("id", &tn_t::Node::id)
        .def_readonly("name", &tn_t::Node::name)
        .def_readonly("indices", &tn_t::Node::indices)
        .def_readonly("tags", &tn_t::Node::tags)
        .def_readonly("contracted", &tn_t::Node::contracted)
        .def_readonly("tensor", &tn_t::Node::tensor);
    py::class_<typename tn_t::Edge>(m, ("TensorNetworkEdge" + s).c_str())
        .def_readonly("dim", &tn_t::Edge::dim)
        .def_readonly("node_ids", &tn_t::Edge::node_ids)
        .def("__eq__", &tn_t::Edge::operator==);
    py::class_<tn_t>(m, ("TensorNetwork" + s).c_str())
        .def(py::init<>())
        .def_property_readonly("index_to_edge_map", &tn_t::GetIndexToEdgeMap)
        .def_property_readonly("tag_to_node_id_map",
                               [](const tn_t &tn) {
                                   std::unordered_map<std::string, std::vector<size_t>> out;
                                   for (const auto &kv : tn.GetTagToNodesMap())
                                       out[kv.first].push_back(kv.second);
                                   return out;
                               })
        .def_property_readonly("nodes", &tn_t::GetNodes)
        .def_property_readonly("path", &tn_t::GetPath)
        .def_property_readonly("num_tensors", &tn_t::NumTensors)
        .def_property_readonly("num_indices", &tn_t::NumIndices)
        .def("add_tensor", &tn_t::AddTensor, py::arg("tensor"),
             py::arg("tags") = std::vector<std::string>())
        .def("slice_indices", &tn_t::SliceIndices, py::arg("indices"), py::arg("value"))
        .def("contract", &tn_t::Contract, py::arg("path") = typename tn_t::Path(),
             py::return_value_policy::copy);
}

template <class T> void BindContractor(py::module_ &m)
{
    using tensor_t = Jet::Tensor<T>;
    using tbc_t = Jet::TaskBasedContractor<tensor_t>;
    py::class_<tbc_t>(m, ("TaskBasedContractor" + Suffix<T>()).c_str())
        .def(py::init<>())
        .def_property_readonly("name_to_tensor_map",
                               [](const tbc_t &t) {
                                   std::unordered_map<std::string, py::object> out;
                                   for (const auto &[name, ptr] : t.GetNameToTensorMap())
                                       out.emplace(name, ptr ? py::cast(*ptr) : py::none());
                                   return out;
                               })
        .def_property_readonly("name_to_parents_map", &tbc_t::GetNameToParentsMap)
        .def_property_readonly("results", &tbc_t::GetResults)
        .def_property_readonly("reduction_result", &tbc_t::GetReductionResult)
        .def_property_readonly("flops", &tbc_t::GetFlops)
        .def_property_readonly("memory", &tbc_t::GetMemory)
        .def("add_contraction_tasks", &tbc_t::AddContractionTasks, py::arg("tn"),
             py::arg("path_info"))
        .def("add_reduction_task", &tbc_t::AddReductionTask)
        .def("add_deletion_tasks", &tbc_t::AddDeletionTasks)
        .def("set_graph_replay", &tbc_t::SetGraphReplay, py::arg("on"))
        .def("set_grouping", &tbc_t::SetGrouping, py::arg("on"))
        .def_property_readonly("has_replay_graph", &tbc_t::HasReplayGraph)
        .def("contract",
             [](tbc_t &t) {
                 py::gil_scoped_release release;
                 t.Contract().get();
             });
}

template <class T> void BindSliced(py::module_ &m)
{
    using sc_t = Jet::SlicedContractor<T>;
    using tn_t = Jet::TensorNetwork<Jet::Tensor<T>>;
    py::class_<sc_t>(m, ("SlicedContractor" + Suffix<T>()).c_str(),
                     "All slices of a sliced network along one path, batched on the GPU.")
        .def(py::init<const tn_t &, const Jet::PathInfo::Path &, const std::vector<std::string> &,
                      int>(),
             py::arg("tn"), py::arg("path"), py::arg("sliced_indices"), py::arg("precision") = 0)
        .def("set_batch_size", &sc_t::SetBatchSize, py::arg("slices_per_batch"))
        .def("set_exponent_hints", &sc_t::SetExponentHints, py::arg("on"))
        .def("set_grouping", &sc_t::SetGrouping, py::arg("on"))
        .def("set_leaf_alternatives", &sc_t::SetLeafAlternatives, py::arg("node_id"),
             py::arg("values"), py::arg("count"))
        .def("contract",
             [](sc_t &s, size_t first, py::object count) {
                 const size_t c = count.is_none() ? SIZE_MAX : count.cast<size_t>();
                 py::gil_scoped_release release;
                 return s.Contract(first, c);
             },
             py::arg("first") = 0, py::arg("count") = py::none())
        .def("profile_chunk",
             [](sc_t &s, size_t first) {
                 std::vector<typename sc_t::ChunkProfileEntry> prof;
                 {
                     py::gil_scoped_release release;
                     prof = s.ProfileChunk(first);
                 }
                 py::list out;
                 for (const auto &e : prof) {
                     py::dict d;
                     d["kind"] = e.kind;
                     d["step"] = e.step;
                     d["batch"] = e.batch;
                     d["m"] = e.m;
                     d["n"] = e.n;
                     d["k"] = e.k;
                     d["ms"] = e.ms;
                     out.append(d);
                 }
                 return out;
             },
             py::arg("first") = 0,
             "Device ms of every gather, contraction and the slice sum of one chunk.")
        .def_property_readonly("batch_size", &sc_t::GetBatchSize)
        .def_property_readonly("num_slices", &sc_t::GetNumSlices)
        .def_property_readonly("result_indices", &sc_t::GetResultIndices)
        .def_property_readonly("result_shape", &sc_t::GetResultShape)
        .def_property_readonly("slice_flops", &sc_t::GetSliceFlops)
        .def_property_readonly("slice_dependent_flops", &sc_t::GetSliceDependentFlops)
        .def_property_readonly("arena_bytes", &sc_t::GetArenaBytes)
        .def("estimate_device_bytes", &sc_t::EstimateDeviceBytes);
}

template <class T> void BindPathInfoCtor(py::class_<Jet::PathInfo> &c)
{
    c.def(py::init<const Jet::TensorNetwork<Jet::Tensor<T>> &, const Jet::PathInfo::Path &>(),
          py::arg("tn"), py::arg("path") = Jet::PathInfo::Path());
}

} // namespace

PYBIND11_MODULE(_jet_bindings, m)
{
    m.doc() = "GB300 Jet host API: tensors, networks, paths and contractors on the GPU.";
    BindTensor<std::complex<float>>(m);
    BindTensor<std::complex<double>>(m);
    BindTensorNetwork<std::complex<float>>(m);
    BindTensorNetwork<std::complex<double>>(m);
    py::class_<Jet::PathStepInfo>(m, "PathStepInfo")
        .def_readonly("id", &Jet::PathStepInfo::id)
        .def_readonly("parent", &Jet::PathStepInfo::parent)
        .def_readonly("children", &Jet::PathStepInfo::children)
        .def_readonly("name", &Jet::PathStepInfo::name)
        .def_readonly("node_indices", &Jet::PathStepInfo::node_indices)
        .def_readonly("tensor_indices", &Jet::PathStepInfo::tensor_indices)
        .def_readonly("tags", &Jet::PathStepInfo::tags)
        .def_readonly("contracted_indices", &Jet::PathStepInfo::contracted_indices)
        .def_property_readonly_static("MISSING_ID",
                                      [](py::object) { return Jet::PathStepInfo::MISSING_ID; });
    py::class_<Jet::PathInfo> pi(m, "PathInfo");
    pi.def(py::init<>())
        .def_property_readonly("index_to_size_map", &Jet::PathInfo::GetIndexSizes)
        .def_property_readonly("num_leaves", &Jet::PathInfo::GetNumLeaves)
        .def_property_readonly("path", &Jet::PathInfo::GetPath)
        .def_property_readonly("steps", &Jet::PathInfo::GetSteps)
        .def("total_flops", &Jet::PathInfo::GetTotalFlops)
        .def("total_memory", &Jet::PathInfo::GetTotalMemory)
        .def("step_flops", &Jet::PathInfo::GetPathStepFlops, py::arg("id"))
        .def("step_memory", &Jet::PathInfo::GetPathStepMemory, py::arg("id"));
    BindPathInfoCtor<std::complex<float>>(pi);
    BindPathInfoCtor<std::complex<double>>(pi);
    BindContractor<std::complex<float>>(m);
    BindContractor<std::complex<double>>(m);
    BindSliced<std::complex<float>>(m);
    BindSliced<std::complex<double>>(m);
    m.def("version", [] { return std::string("0.2.3-gb300"); });
    m.def("set_precision", &Jet::Gpu::SetPrecision, py::arg("precision"),
          "ContractTensors arithmetic for complex64: 0 plain FP32, 1 TF32x3, 2 auto, 3 BF16x3, "
          "4 FP16x3, 5 tuned (the autotuner's fastest per shape).");
    m.def("get_precision", &Jet::Gpu::GetPrecision);
    py::register_exception<Jet::Exception>(m, "JetException", PyExc_RuntimeError);
}
