// TaskBasedContractor's DOT dump (reference: TaskBasedContractor.hpp:429-452).
// Host only: builds the tasks of two networks that share a prefix, adds the
// reduction and deletion tasks, and prints the graph. Run by
// tests/test_cuda_tensor.py, which checks the nodes and edges.
#include <complex>
#include <iostream>

#include "Jet.hpp"

using namespace Jet;
using T = std::complex<float>;

int main()
{
    // Two 3-tensor chains A(i,j) B(j,k) C(k) with different C: the first
    // step (A.B) is shared by name, the second differs.
    TaskBasedContractor<Tensor<T>> tbc;
    for (int net = 0; net < 2; ++net) {
        TensorNetwork<Tensor<T>> tn;
        tn.AddTensor(Tensor<T>({"i", "j"}, {2, 2}, {1, 2, 3, 4}), {"A"});
        tn.AddTensor(Tensor<T>({"j", "k"}, {2, 2}, {1, 0, 0, 1}), {"B"});
        tn.AddTensor(Tensor<T>({"k"}, {2}, {T(1.0f + net), 0}), {"C" + std::to_string(net)});
        PathInfo info(tn, {{0, 1}, {2, 3}});
        std::cout << "shared " << tbc.AddContractionTasks(tn, info) << "\n";
    }
    tbc.AddReductionTask();
    tbc.AddDeletionTasks();
    std::cout << tbc;
    return 0;
}
