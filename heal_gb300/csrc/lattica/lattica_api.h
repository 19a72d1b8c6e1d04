// lattica_api.h — the HEAL hardware API (namespace lattica_hw_api) as this
// backend implements it.
//
// The declarations restate HEAL's include/ headers signature for signature
// (device_memory.h:24-39, memory_virtual_ops.h:39-86, contiguous.h:19-20,
// modop.h:47-134, axis_modsum.h:24-30, g_decomposition.h:24-30,
// ntt.h:31-52, permute.h:33-40), so code written against HEAL links against
// this library unchanged: the explicit instantiations for int32_t, int64_t
// (and double for the memory ops) have the same mangled names.
//
// DeviceTensor<T> is the vendor-defined tensor of device_memory.h:11-16; here
// its buffer is HBM from the backend's stream-ordered pool and every method
// HEAL declares (reshape, print, print_metadata) is provided.
#pragma once
#include <ATen/core/Tensor.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "../../../include/heal_gb300.h"

template <typename T>
struct DeviceTensor {
  std::vector<int64_t> dims;
  std::vector<int64_t> strides;  // in elements; 0 on broadcast axes
  std::shared_ptr<void> data;    // HBM allocation, released with heal_free
  int64_t offset = 0;            // element (0,...,0) relative to data (slices)

  DeviceTensor(const std::vector<int64_t> &dims, const std::vector<int64_t> &strides, std::shared_ptr<void> data,
               int64_t offset = 0);

  void reshape(const std::vector<int64_t> &new_dims);
  void print() const;
  void print_metadata() const;
  bool is_contiguous() const;
  heal_tensor desc() const;  // the C-ABI view of this tensor
  void assign(const heal_tensor &d);  // takes dims/strides/offset from a view of the same buffer
};

namespace lattica_hw_api {

template <typename T>
std::shared_ptr<DeviceTensor<T>> allocate_on_hardware(const std::vector<int64_t> &dims);
template <typename T>
std::shared_ptr<DeviceTensor<T>> host_to_device(const at::Tensor &tensor);
template <typename T>
at::Tensor device_to_host(const std::shared_ptr<DeviceTensor<T>> &memory);

template <typename T>
std::shared_ptr<DeviceTensor<T>> expand(const std::shared_ptr<DeviceTensor<T>> &tensor, int64_t axis, int64_t repeats);
template <typename T>
std::shared_ptr<DeviceTensor<T>> squeeze(const std::shared_ptr<DeviceTensor<T>> &tensor, int64_t axis);
template <typename T>
std::shared_ptr<DeviceTensor<T>> unsqueeze(const std::shared_ptr<DeviceTensor<T>> &tensor, int64_t axis);
template <typename T>
std::shared_ptr<DeviceTensor<T>> make_contiguous(const std::shared_ptr<DeviceTensor<T>> &tensor);

template <typename T>
void modmul_ttt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                const std::shared_ptr<DeviceTensor<T>> &p, std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modmul_ttc(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b, T p_scalar,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modmul_tct(const std::shared_ptr<DeviceTensor<T>> &a, T b_scalar, const std::shared_ptr<DeviceTensor<T>> &p,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modmul_tcc(const std::shared_ptr<DeviceTensor<T>> &a, T b_scalar, T p_scalar,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modsum_ttt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                const std::shared_ptr<DeviceTensor<T>> &p, std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modsum_ttc(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b, T p_scalar,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modsum_tct(const std::shared_ptr<DeviceTensor<T>> &a, T b_scalar, const std::shared_ptr<DeviceTensor<T>> &p,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modsum_tcc(const std::shared_ptr<DeviceTensor<T>> &a, T b_scalar, T p_scalar,
                std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void mod_tt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
            std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void mod_tc(const std::shared_ptr<DeviceTensor<T>> &a, int64_t b_scalar, std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void mod_ct(int64_t a_scalar, const std::shared_ptr<DeviceTensor<T>> &b, std::shared_ptr<DeviceTensor<T>> &result);

template <typename T>
void axis_modsum(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
                 std::shared_ptr<DeviceTensor<T>> &result, int64_t axis);

template <typename T>
void g_decomposition(const std::shared_ptr<DeviceTensor<T>> &a, std::shared_ptr<DeviceTensor<T>> &result,
                     size_t power, size_t base_bits);

template <typename T>
void ntt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
         const std::shared_ptr<DeviceTensor<T>> &perm, const std::shared_ptr<DeviceTensor<T>> &twiddles,
         const std::shared_ptr<DeviceTensor<T>> &log2p_list, const std::shared_ptr<DeviceTensor<T>> &mu_list,
         std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void intt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
          const std::shared_ptr<DeviceTensor<T>> &perm, const std::shared_ptr<DeviceTensor<T>> &inv_twiddles,
          const std::shared_ptr<DeviceTensor<T>> &m_inv, const std::shared_ptr<DeviceTensor<T>> &log2p_list,
          const std::shared_ptr<DeviceTensor<T>> &mu_list, std::shared_ptr<DeviceTensor<T>> &result);

template <typename T>
void permute(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &perms,
             std::shared_ptr<DeviceTensor<T>> &result, int64_t elementwise_axis, int64_t perm_axis);

// ---- extensions (no HEAL declaration; named by the runtime's
// DeviceDispatcher, python_execution/lattica_heal_runtime/device_interface.py)
template <typename T>
void modneg_tt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
               std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
void modneg_tc(const std::shared_ptr<DeviceTensor<T>> &a, T p_scalar, std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
std::shared_ptr<DeviceTensor<T>> moveaxis(const std::shared_ptr<DeviceTensor<T>> &tensor, int64_t src, int64_t dst);
// result = axis_modsum(modmul(a', b, p), axis), a' = a gathered by perms (may
// be null) along perm_axis: DeviceDispatcher.modmul_axis_sum
// (device_interface.py:67-68); see heal_modmul_axis_sum.
template <typename T>
void modmul_axis_sum(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                     const std::shared_ptr<DeviceTensor<T>> &p, const std::shared_ptr<DeviceTensor<T>> &perms,
                     int64_t perm_axis, std::shared_ptr<DeviceTensor<T>> &result, int64_t axis);
// result = ntt(reshape(g_decomposition(a, power, base_bits), [l, m, r, k * power]),
// p, perm, twiddles) in one call (an extension; see heal_g_decomposition_ntt).
template <typename T>
void g_decomposition_ntt(const std::shared_ptr<DeviceTensor<T>> &a, size_t power, size_t base_bits,
                         const std::shared_ptr<DeviceTensor<T>> &p, const std::shared_ptr<DeviceTensor<T>> &perm,
                         const std::shared_ptr<DeviceTensor<T>> &twiddles, std::shared_ptr<DeviceTensor<T>> &result);
// result = permute(axis_modsum(modmul(a, b, p), axis), perms, elementwise_axis,
// perm_axis) in one pass (an extension; see heal_modmul_axis_sum_permute).
template <typename T>
void modmul_axis_sum_permute(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                             const std::shared_ptr<DeviceTensor<T>> &p, int64_t axis,
                             const std::shared_ptr<DeviceTensor<T>> &perms, int64_t elementwise_axis,
                             int64_t perm_axis, std::shared_ptr<DeviceTensor<T>> &result);
template <typename T>
std::shared_ptr<DeviceTensor<T>> get_slice(const std::shared_ptr<DeviceTensor<T>> &tensor, int64_t axis,
                                           int64_t start, int64_t stop, int64_t step);
void synchronize();

}  // namespace lattica_hw_api
