// py_bindings.cpp — the `lattica_hw` Python module over the GB300 backend.
//
// Same module name, class names and function names as HEAL's
// example_impl/py_bindings.cpp:87-133 (DeviceTensor{32,64,float64};
// <op>_{32,64,float64}), so python_execution/lattica_heal_runtime/py_wrapper.py
// imports it unchanged.  Added: mod_*, modneg_*, moveaxis_*, get_slice_*, view_*,
// modmul_axis_sum_*, g_decomposition_ntt_*, modmul_axis_sum_permute_* and synchronize(), which HEAL's
// module does not export.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <torch/extension.h>

#include "lattica_api.h"

namespace py = pybind11;
using namespace lattica_hw_api;

template <typename T>
static void bind_tensor(py::module_ &m, const std::string &sfx) {
  using D = DeviceTensor<T>;
  py::class_<D, std::shared_ptr<D>>(m, ("DeviceTensor" + sfx).c_str())
      .def("print", &D::print)
      .def("print_metadata", &D::print_metadata)
      .def("reshape", &D::reshape)
      .def_property_readonly("dims", [](const D &t) { return t.dims; })
      .def_property_readonly("strides", [](const D &t) { return t.strides; })
      .def("data_ptr", [](const D &t) { return (uintptr_t)t.desc().data; });
  m.def(("allocate_on_hardware_" + sfx).c_str(), &allocate_on_hardware<T>, py::arg("dims"));
  m.def(("host_to_device_" + sfx).c_str(), &host_to_device<T>, py::arg("tensor"));
  m.def(("device_to_host_" + sfx).c_str(), &device_to_host<T>, py::arg("device_mem"));
  m.def(("expand_" + sfx).c_str(), &expand<T>, py::arg("tensor"), py::arg("axis"), py::arg("repeats"));
  m.def(("squeeze_" + sfx).c_str(), &squeeze<T>, py::arg("tensor"), py::arg("axis"));
  m.def(("unsqueeze_" + sfx).c_str(), &unsqueeze<T>, py::arg("tensor"), py::arg("axis"));
  m.def(("make_contiguous_" + sfx).c_str(), &make_contiguous<T>, py::arg("tensor"));
  m.def(("moveaxis_" + sfx).c_str(), &moveaxis<T>, py::arg("tensor"), py::arg("source"), py::arg("destination"));
  m.def(("get_slice_" + sfx).c_str(), &get_slice<T>, py::arg("tensor"), py::arg("axis"), py::arg("start"),
        py::arg("stop"), py::arg("step") = 1);
  // a new view object of the same buffer, dims and strides
  m.def(("view_" + sfx).c_str(), [](const std::shared_ptr<D> &t) {
    if (!t) throw std::invalid_argument("tensor pointer must not be null.");
    return std::make_shared<D>(*t);
  }, py::arg("tensor"));
}

template <typename T>
static void bind_compute(py::module_ &m, const std::string &sfx) {
  m.def(("modmul_ttt_" + sfx).c_str(), &modmul_ttt<T>);
  m.def(("modmul_ttc_" + sfx).c_str(), &modmul_ttc<T>);
  m.def(("modmul_tct_" + sfx).c_str(), &modmul_tct<T>);
  m.def(("modmul_tcc_" + sfx).c_str(), &modmul_tcc<T>);
  m.def(("modsum_ttt_" + sfx).c_str(), &modsum_ttt<T>);
  m.def(("modsum_ttc_" + sfx).c_str(), &modsum_ttc<T>);
  m.def(("modsum_tct_" + sfx).c_str(), &modsum_tct<T>);
  m.def(("modsum_tcc_" + sfx).c_str(), &modsum_tcc<T>);
  m.def(("mod_tt_" + sfx).c_str(), &mod_tt<T>);
  m.def(("mod_tc_" + sfx).c_str(), &mod_tc<T>);
  m.def(("mod_ct_" + sfx).c_str(), &mod_ct<T>);
  m.def(("modneg_tt_" + sfx).c_str(), &modneg_tt<T>);
  m.def(("modneg_tc_" + sfx).c_str(), &modneg_tc<T>);
  m.def(("axis_modsum_" + sfx).c_str(), &axis_modsum<T>);
  m.def(("g_decomposition_" + sfx).c_str(), &g_decomposition<T>, py::arg("a"), py::arg("result"), py::arg("power"),
        py::arg("base_bits"));
  m.def(("ntt_" + sfx).c_str(), &ntt<T>);
  m.def(("intt_" + sfx).c_str(), &intt<T>);
  m.def(("permute_" + sfx).c_str(), &permute<T>);
  m.def(("modmul_axis_sum_" + sfx).c_str(), &modmul_axis_sum<T>, py::arg("a"), py::arg("b"), py::arg("p"),
        py::arg("perms"), py::arg("perm_axis"), py::arg("result"), py::arg("axis"));
  m.def(("g_decomposition_ntt_" + sfx).c_str(), &g_decomposition_ntt<T>, py::arg("a"), py::arg("power"),
        py::arg("base_bits"), py::arg("p"), py::arg("perm"), py::arg("twiddles"), py::arg("result"));
  m.def(("modmul_axis_sum_permute_" + sfx).c_str(), &modmul_axis_sum_permute<T>, py::arg("a"), py::arg("b"),
        py::arg("p"), py::arg("axis"), py::arg("perms"), py::arg("elementwise_axis"), py::arg("perm_axis"),
        py::arg("result"));
}

PYBIND11_MODULE(lattica_hw, m) {
  m.doc() = "HEAL hardware API on the GB300 backend";
  bind_tensor<int32_t>(m, "32");
  bind_tensor<int64_t>(m, "64");
  bind_tensor<double>(m, "float64");
  bind_compute<int32_t>(m, "32");
  bind_compute<int64_t>(m, "64");
  m.def("synchronize", &synchronize);
  m.def("kernel_launch_count", []() { return heal_kernel_launch_count(); });
}
