// Python binding for the reference's fairnr/clib/src/octree.cpp compiled as a
// CPU torch extension by oracle/build_ref.py. TEST INFRASTRUCTURE ONLY.
#include <torch/extension.h>
#include <tuple>
std::tuple<at::Tensor, at::Tensor> build_octree(at::Tensor center, at::Tensor points, int depth);
PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) { m.def("build_octree", &build_octree); }
