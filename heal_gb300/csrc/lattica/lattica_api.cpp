// lattica_api.cpp — HEAL's lattica_hw_api templates over the C ABI.
//
// Every function validates through the C ABI (which reproduces the checks
// and messages of example_impl) and turns a failing status into the C++
// exception HEAL's sample throws for it.  Compute calls are stream-ordered;
// device_to_host and print wait for all earlier work, so a HEAL caller sees
// the same results as with the synchronous sample implementation.
#include "lattica_api.h"

#include <ATen/Functions.h>

#include <functional>
#include <iostream>
#include <new>
#include <stdexcept>
#include <string>
#include <typeinfo>

namespace {

template <typename T>
constexpr int dtype_of();
template <>
constexpr int dtype_of<int32_t>() {
  return HEAL_INT32;
}
template <>
constexpr int dtype_of<int64_t>() {
  return HEAL_INT64;
}
template <>
constexpr int dtype_of<double>() {
  return HEAL_FLOAT64;
}

void check(int rc) {
  if (rc == HEAL_OK) return;
  std::string msg = heal_last_error();
  switch (rc) {
    case HEAL_ERR_INVALID_ARGUMENT:
      throw std::invalid_argument(msg);
    case HEAL_ERR_OUT_OF_RANGE:
      throw std::out_of_range(msg);
    case HEAL_ERR_BAD_ALLOC:
      throw std::bad_alloc();
    default:
      throw std::runtime_error(msg);
  }
}

std::shared_ptr<void> device_buffer(size_t bytes, bool zero) {
  void *p = nullptr;
  check(heal_alloc(bytes, zero ? 1 : 0, &p));
  return std::shared_ptr<void>(p, [](void *q) { heal_free(q); });
}

std::vector<int64_t> rowmajor(const std::vector<int64_t> &dims) {
  std::vector<int64_t> s(dims.size());
  int64_t st = 1;
  for (int i = (int)dims.size() - 1; i >= 0; --i) {
    s[i] = st;
    st *= dims[i];
  }
  return s;
}

int64_t count(const std::vector<int64_t> &dims) {
  int64_t n = 1;
  for (int64_t d : dims) n *= d;
  return n;
}

// elements spanned by a view (device_memory_impl.cpp:19-23), 0 when empty
int64_t span(const std::vector<int64_t> &dims, const std::vector<int64_t> &strides) {
  if (count(dims) == 0) return 0;
  int64_t s = 1;
  for (size_t i = 0; i < dims.size(); ++i) s += (dims[i] - 1) * strides[i];
  return s;
}

template <typename T>
const heal_tensor *opt(const std::shared_ptr<DeviceTensor<T>> &t, heal_tensor &slot) {
  if (!t) return nullptr;
  slot = t->desc();
  return &slot;
}

template <typename T>
heal_tensor need(const std::shared_ptr<DeviceTensor<T>> &t, const char *label) {
  if (!t) throw std::invalid_argument(std::string(label) + " pointer must not be null.");
  return t->desc();
}

}  // namespace

// ============================================================ DeviceTensor
template <typename T>
DeviceTensor<T>::DeviceTensor(const std::vector<int64_t> &dims, const std::vector<int64_t> &strides,
                              std::shared_ptr<void> data, int64_t offset)
    : dims(dims), strides(strides), data(std::move(data)), offset(offset) {}

template <typename T>
heal_tensor DeviceTensor<T>::desc() const {
  if (dims.size() > HEAL_MAX_DIMS) throw std::invalid_argument("DeviceTensor: more than 8 dimensions");
  heal_tensor d;
  d.data = data ? (void *)((char *)data.get() + offset * (int64_t)sizeof(T)) : nullptr;
  d.dtype = dtype_of<T>();
  d.ndim = (int32_t)dims.size();
  for (int i = 0; i < HEAL_MAX_DIMS; ++i) {
    d.dims[i] = i < d.ndim ? dims[i] : 1;
    d.strides[i] = i < d.ndim ? strides[i] : 0;
  }
  return d;
}

template <typename T>
void DeviceTensor<T>::assign(const heal_tensor &d) {
  dims.assign(d.dims, d.dims + d.ndim);
  strides.assign(d.strides, d.strides + d.ndim);
  if (data && d.data) offset = ((char *)d.data - (char *)data.get()) / (int64_t)sizeof(T);
}

template <typename T>
void DeviceTensor<T>::reshape(const std::vector<int64_t> &new_dims) {
  heal_tensor d = desc();
  if (new_dims.size() > HEAL_MAX_DIMS) throw std::invalid_argument("reshape: more than 8 dimensions");
  check(heal_tensor_reshape(&d, (int32_t)new_dims.size(), new_dims.data()));
  assign(d);
}

template <typename T>
bool DeviceTensor<T>::is_contiguous() const {
  // device_memory_impl.cpp:31-40
  int64_t expected = 1;
  for (int i = (int)dims.size() - 1; i >= 0; --i) {
    if (dims[i] == 1) continue;
    if (strides[i] != expected) return false;
    expected *= dims[i];
  }
  return true;
}

template <typename T>
void DeviceTensor<T>::print_metadata() const {
  // device_memory_impl.cpp:156-164
  std::cout << "DeviceTensor<" << typeid(T).name() << "> ";
  std::cout << "Shape: [";
  for (auto d : dims) std::cout << d << " ";
  std::cout << "]  Strides: [";
  for (auto s : strides) std::cout << s << " ";
  std::cout << "]\n\n" << std::flush;
}

template <typename T>
void DeviceTensor<T>::print() const {
  // device_memory_impl.cpp:126-154, reading the elements back from HBM
  std::cout << "DeviceTensor<" << typeid(T).name() << "> ";
  std::cout << "Shape: [";
  for (auto d : dims) std::cout << d << " ";
  std::cout << "]  Strides: [";
  for (auto s : strides) std::cout << s << " ";
  std::cout << "]\n";
  std::cout << "]\nData: ";
  const int64_t n = span(dims, strides);
  std::vector<T> host((size_t)std::max<int64_t>(n, 1));
  heal_tensor d = desc();
  check(heal_d2h(host.data(), d.data, (size_t)n * sizeof(T)));
  std::vector<int64_t> idx(dims.size(), 0);
  std::function<void(size_t)> rec = [&](size_t dim) {
    if (dim == dims.size()) {
      int64_t off = 0;
      for (size_t i = 0; i < dims.size(); ++i) off += idx[i] * strides[i];
      std::cout << host[(size_t)off];
      return;
    }
    std::cout << "{";
    for (int64_t i = 0; i < dims[dim]; ++i) {
      idx[dim] = i;
      if (i > 0) std::cout << ", ";
      rec(dim + 1);
    }
    std::cout << "}";
  };
  rec(0);
  std::cout << "\n\n" << std::flush;
}

template struct DeviceTensor<int32_t>;
template struct DeviceTensor<int64_t>;
template struct DeviceTensor<double>;

namespace lattica_hw_api {

// ============================================================ memory
template <typename T>
std::shared_ptr<DeviceTensor<T>> allocate_on_hardware(const std::vector<int64_t> &dims) {
  // device_memory_impl.cpp:168-179: zeroed, row-major
  for (int64_t d : dims)
    if (d < 0) throw std::invalid_argument("allocate_on_hardware: negative dimension");
  int64_t n = count(dims);
  auto buf = n ? device_buffer((size_t)n * sizeof(T), true) : std::shared_ptr<void>();
  return std::make_shared<DeviceTensor<T>>(dims, rowmajor(dims), buf);
}

template <typename T>
std::shared_ptr<DeviceTensor<T>> host_to_device(const at::Tensor &tensor) {
  // device_memory_impl.cpp:181-190: same dtype, the source's strides kept
  if (tensor.scalar_type() != c10::CppTypeToScalarType<T>::value)
    throw std::runtime_error("Tensor dtype does not match template parameter T.");
  std::vector<int64_t> dims(tensor.sizes().begin(), tensor.sizes().end());
  std::vector<int64_t> strides(tensor.strides().begin(), tensor.strides().end());
  for (int64_t s : strides)
    if (s < 0) throw std::invalid_argument("host_to_device: negative strides are not supported");
  int64_t n = span(dims, strides);
  std::shared_ptr<void> buf;
  if (n) {
    buf = device_buffer((size_t)n * sizeof(T), false);
    check(heal_h2d(buf.get(), tensor.data_ptr(), (size_t)n * sizeof(T)));
  }
  return std::make_shared<DeviceTensor<T>>(dims, strides, buf);
}

template <typename T>
at::Tensor device_to_host(const std::shared_ptr<DeviceTensor<T>> &memory) {
  // device_memory_impl.cpp:192-202: from_blob(dims, strides).clone()
  heal_tensor d = need(memory, "memory");
  auto opts = at::TensorOptions().dtype(c10::CppTypeToScalarType<T>::value);
  int64_t n = span(memory->dims, memory->strides);
  if (n == 0) {
    check(heal_synchronize());
    return at::empty(memory->dims, opts);
  }
  at::Tensor host = at::empty({n}, opts);
  check(heal_d2h(host.data_ptr(), d.data, (size_t)n * sizeof(T)));
  return at::from_blob(host.data_ptr(), memory->dims, memory->strides, opts).clone();
}

// ============================================================ virtual ops
template <typename T>
static std::shared_ptr<DeviceTensor<T>> meta(const std::shared_ptr<DeviceTensor<T>> &t,
                                             const std::function<int(heal_tensor *)> &f) {
  heal_tensor d = need(t, "tensor");
  check(f(&d));
  t->assign(d);
  return t;
}

template <typename T>
std::shared_ptr<DeviceTensor<T>> expand(const std::shared_ptr<DeviceTensor<T>> &t, int64_t axis, int64_t repeats) {
  return meta<T>(t, [&](heal_tensor *d) { return heal_tensor_expand(d, axis, repeats); });
}
template <typename T>
std::shared_ptr<DeviceTensor<T>> squeeze(const std::shared_ptr<DeviceTensor<T>> &t, int64_t axis) {
  return meta<T>(t, [&](heal_tensor *d) { return heal_tensor_squeeze(d, axis); });
}
template <typename T>
std::shared_ptr<DeviceTensor<T>> unsqueeze(const std::shared_ptr<DeviceTensor<T>> &t, int64_t axis) {
  return meta<T>(t, [&](heal_tensor *d) { return heal_tensor_unsqueeze(d, axis); });
}
template <typename T>
std::shared_ptr<DeviceTensor<T>> moveaxis(const std::shared_ptr<DeviceTensor<T>> &t, int64_t src, int64_t dst) {
  return meta<T>(t, [&](heal_tensor *d) { return heal_tensor_moveaxis(d, src, dst); });
}
template <typename T>
std::shared_ptr<DeviceTensor<T>> get_slice(const std::shared_ptr<DeviceTensor<T>> &t, int64_t axis, int64_t start,
                                           int64_t stop, int64_t step) {
  // a new view object sharing the buffer (the source view is left as is)
  if (!t) throw std::invalid_argument("tensor pointer must not be null.");
  auto v = std::make_shared<DeviceTensor<T>>(*t);
  return meta<T>(v, [&](heal_tensor *d) { return heal_tensor_slice(d, axis, start, stop, step); });
}

template <typename T>
std::shared_ptr<DeviceTensor<T>> make_contiguous(const std::shared_ptr<DeviceTensor<T>> &t) {
  // contiguous_impl.cpp:9-52: same object; new dense buffer if strided
  heal_tensor src = need(t, "tensor");
  if (t->is_contiguous()) return t;
  int64_t n = count(t->dims);
  auto buf = n ? device_buffer((size_t)n * sizeof(T), false) : std::shared_ptr<void>();
  auto dense = rowmajor(t->dims);
  DeviceTensor<T> out(t->dims, dense, buf);
  heal_tensor dst = out.desc();
  check(heal_copy_strided(&src, &dst));
  t->data = buf;
  t->offset = 0;
  t->strides = dense;
  return t;
}

// ============================================================ arithmetic
#define HEAL_TTT(NAME, CFN)                                                                                 \
  template <typename T>                                                                                     \
  void NAME(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,          \
            const std::shared_ptr<DeviceTensor<T>> &p, std::shared_ptr<DeviceTensor<T>> &result) {         \
    heal_tensor A = need(a, "a"), B = need(b, "b"), P = need(p, "p"), R = need(result, "result");         \
    check(CFN(&A, &B, &P, &R));                                                                             \
  }
#define HEAL_TTC(NAME, CFN)                                                                                 \
  template <typename T>                                                                                     \
  void NAME(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b, T p,     \
            std::shared_ptr<DeviceTensor<T>> &result) {                                                    \
    heal_tensor A = need(a, "a"), B = need(b, "b"), R = need(result, "result");                           \
    check(CFN(&A, &B, (int64_t)p, &R));                                                                     \
  }
#define HEAL_TCT(NAME, CFN)                                                                                 \
  template <typename T>                                                                                     \
  void NAME(const std::shared_ptr<DeviceTensor<T>> &a, T b, const std::shared_ptr<DeviceTensor<T>> &p,     \
            std::shared_ptr<DeviceTensor<T>> &result) {                                                    \
    heal_tensor A = need(a, "a"), P = need(p, "p"), R = need(result, "result");                           \
    check(CFN(&A, (int64_t)b, &P, &R));                                                                     \
  }
#define HEAL_TCC(NAME, CFN)                                                                                  \
  template <typename T>                                                                                      \
  void NAME(const std::shared_ptr<DeviceTensor<T>> &a, T b, T p, std::shared_ptr<DeviceTensor<T>> &result) { \
    heal_tensor A = need(a, "a"), R = need(result, "result");                                              \
    check(CFN(&A, (int64_t)b, (int64_t)p, &R));                                                              \
  }

HEAL_TTT(modmul_ttt, heal_modmul_ttt)
HEAL_TTC(modmul_ttc, heal_modmul_ttc)
HEAL_TCT(modmul_tct, heal_modmul_tct)
HEAL_TCC(modmul_tcc, heal_modmul_tcc)
HEAL_TTT(modsum_ttt, heal_modsum_ttt)
HEAL_TTC(modsum_ttc, heal_modsum_ttc)
HEAL_TCT(modsum_tct, heal_modsum_tct)
HEAL_TCC(modsum_tcc, heal_modsum_tcc)

template <typename T>
void mod_tt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
            std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), B = need(b, "b"), R = need(result, "result");
  check(heal_mod_tt(&A, &B, &R));
}
template <typename T>
void mod_tc(const std::shared_ptr<DeviceTensor<T>> &a, int64_t b, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), R = need(result, "result");
  check(heal_mod_tc(&A, b, &R));
}
template <typename T>
void mod_ct(int64_t a, const std::shared_ptr<DeviceTensor<T>> &b, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor B = need(b, "b"), R = need(result, "result");
  check(heal_mod_ct(a, &B, &R));
}
template <typename T>
void modneg_tt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
               std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), P = need(p, "p"), R = need(result, "result");
  check(heal_modneg_tt(&A, &P, &R));
}
template <typename T>
void modneg_tc(const std::shared_ptr<DeviceTensor<T>> &a, T p, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), R = need(result, "result");
  check(heal_modneg_tc(&A, (int64_t)p, &R));
}

template <typename T>
void axis_modsum(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
                 std::shared_ptr<DeviceTensor<T>> &result, int64_t axis) {
  heal_tensor A = need(a, "a"), P = need(p, "p"), R = need(result, "result");
  check(heal_axis_modsum(&A, &P, &R, axis));
}

template <typename T>
void g_decomposition(const std::shared_ptr<DeviceTensor<T>> &a, std::shared_ptr<DeviceTensor<T>> &result,
                     size_t power, size_t base_bits) {
  heal_tensor A = need(a, "a"), R = need(result, "result");
  check(heal_g_decomposition(&A, &R, (uint64_t)power, (uint64_t)base_bits));
}

template <typename T>
void ntt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
         const std::shared_ptr<DeviceTensor<T>> &perm, const std::shared_ptr<DeviceTensor<T>> &twiddles,
         const std::shared_ptr<DeviceTensor<T>> &log2p_list, const std::shared_ptr<DeviceTensor<T>> &mu_list,
         std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), P = need(p, "p"), PM = need(perm, "perm"), TW = need(twiddles, "twiddles"),
              R = need(result, "result"), L2, MU;
  check(heal_ntt(&A, &P, &PM, &TW, opt(log2p_list, L2), opt(mu_list, MU), &R));
}

template <typename T>
void intt(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &p,
          const std::shared_ptr<DeviceTensor<T>> &perm, const std::shared_ptr<DeviceTensor<T>> &inv_twiddles,
          const std::shared_ptr<DeviceTensor<T>> &m_inv, const std::shared_ptr<DeviceTensor<T>> &log2p_list,
          const std::shared_ptr<DeviceTensor<T>> &mu_list, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), P = need(p, "p"), PM = need(perm, "perm"),
              TW = need(inv_twiddles, "inv_twiddles"), R = need(result, "result"), MI, L2, MU;
  check(heal_intt(&A, &P, &PM, &TW, opt(m_inv, MI), opt(log2p_list, L2), opt(mu_list, MU), &R));
}

template <typename T>
void permute(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &perms,
             std::shared_ptr<DeviceTensor<T>> &result, int64_t elementwise_axis, int64_t perm_axis) {
  heal_tensor A = need(a, "a"), PM = need(perms, "perms"), R = need(result, "result");
  check(heal_permute(&A, &PM, &R, elementwise_axis, perm_axis));
}

template <typename T>
void modmul_axis_sum(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                     const std::shared_ptr<DeviceTensor<T>> &p, const std::shared_ptr<DeviceTensor<T>> &perms,
                     int64_t perm_axis, std::shared_ptr<DeviceTensor<T>> &result, int64_t axis) {
  heal_tensor A = need(a, "a"), B = need(b, "b"), P = need(p, "p"), R = need(result, "result");
  heal_tensor PM;
  if (perms) PM = perms->desc();
  check(heal_modmul_axis_sum(&A, &B, &P, perms ? &PM : nullptr, perm_axis, &R, axis));
}

template <typename T>
void modmul_axis_sum_permute(const std::shared_ptr<DeviceTensor<T>> &a, const std::shared_ptr<DeviceTensor<T>> &b,
                             const std::shared_ptr<DeviceTensor<T>> &p, int64_t axis,
                             const std::shared_ptr<DeviceTensor<T>> &perms, int64_t elementwise_axis,
                             int64_t perm_axis, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), B = need(b, "b"), P = need(p, "p"), PM = need(perms, "perms"),
              R = need(result, "result");
  check(heal_modmul_axis_sum_permute(&A, &B, &P, axis, &PM, elementwise_axis, perm_axis, &R));
}

template <typename T>
void g_decomposition_ntt(const std::shared_ptr<DeviceTensor<T>> &a, size_t power, size_t base_bits,
                         const std::shared_ptr<DeviceTensor<T>> &p, const std::shared_ptr<DeviceTensor<T>> &perm,
                         const std::shared_ptr<DeviceTensor<T>> &twiddles, std::shared_ptr<DeviceTensor<T>> &result) {
  heal_tensor A = need(a, "a"), P = need(p, "p"), PM = need(perm, "perm"), TW = need(twiddles, "twiddles"),
              R = need(result, "result");
  check(heal_g_decomposition_ntt(&A, (int64_t)power, (int64_t)base_bits, &P, &PM, &TW, &R));
}

void synchronize() { check(heal_synchronize()); }

// ============================================================ instantiations
#define HEAL_MEMORY(T)                                                                                           \
  template std::shared_ptr<DeviceTensor<T>> allocate_on_hardware<T>(const std::vector<int64_t> &);              \
  template std::shared_ptr<DeviceTensor<T>> host_to_device<T>(const at::Tensor &);                             \
  template at::Tensor device_to_host<T>(const std::shared_ptr<DeviceTensor<T>> &);                             \
  template std::shared_ptr<DeviceTensor<T>> expand<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t, int64_t); \
  template std::shared_ptr<DeviceTensor<T>> squeeze<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t);     \
  template std::shared_ptr<DeviceTensor<T>> unsqueeze<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t);   \
  template std::shared_ptr<DeviceTensor<T>> moveaxis<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t, int64_t); \
  template std::shared_ptr<DeviceTensor<T>> get_slice<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t, int64_t, \
                                                         int64_t, int64_t);                                     \
  template std::shared_ptr<DeviceTensor<T>> make_contiguous<T>(const std::shared_ptr<DeviceTensor<T>> &);

#define HEAL_COMPUTE(T)                                                                                            \
  template void modmul_ttt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                              const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &);     \
  template void modmul_ttc<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                              T, std::shared_ptr<DeviceTensor<T>> &);                                            \
  template void modmul_tct<T>(const std::shared_ptr<DeviceTensor<T>> &, T, const std::shared_ptr<DeviceTensor<T>> &, \
                              std::shared_ptr<DeviceTensor<T>> &);                                               \
  template void modmul_tcc<T>(const std::shared_ptr<DeviceTensor<T>> &, T, T, std::shared_ptr<DeviceTensor<T>> &); \
  template void modsum_ttt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                              const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &);     \
  template void modsum_ttc<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                              T, std::shared_ptr<DeviceTensor<T>> &);                                            \
  template void modsum_tct<T>(const std::shared_ptr<DeviceTensor<T>> &, T, const std::shared_ptr<DeviceTensor<T>> &, \
                              std::shared_ptr<DeviceTensor<T>> &);                                               \
  template void modsum_tcc<T>(const std::shared_ptr<DeviceTensor<T>> &, T, T, std::shared_ptr<DeviceTensor<T>> &); \
  template void mod_tt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,     \
                          std::shared_ptr<DeviceTensor<T>> &);                                                   \
  template void mod_tc<T>(const std::shared_ptr<DeviceTensor<T>> &, int64_t, std::shared_ptr<DeviceTensor<T>> &); \
  template void mod_ct<T>(int64_t, const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &); \
  template void modneg_tt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,  \
                             std::shared_ptr<DeviceTensor<T>> &);                                                \
  template void modneg_tc<T>(const std::shared_ptr<DeviceTensor<T>> &, T, std::shared_ptr<DeviceTensor<T>> &);    \
  template void modmul_axis_sum<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                                   const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                                   int64_t, std::shared_ptr<DeviceTensor<T>> &, int64_t);                           \
  template void g_decomposition_ntt<T>(const std::shared_ptr<DeviceTensor<T>> &, size_t, size_t,                \
                                       const std::shared_ptr<DeviceTensor<T>> &,                                  \
                                       const std::shared_ptr<DeviceTensor<T>> &,                                  \
                                       const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &); \
  template void modmul_axis_sum_permute<T>(const std::shared_ptr<DeviceTensor<T>> &,                              \
                                           const std::shared_ptr<DeviceTensor<T>> &,                              \
                                           const std::shared_ptr<DeviceTensor<T>> &, int64_t,                     \
                                           const std::shared_ptr<DeviceTensor<T>> &, int64_t, int64_t,            \
                                           std::shared_ptr<DeviceTensor<T>> &);                                   \
  template void axis_modsum<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &, \
                               std::shared_ptr<DeviceTensor<T>> &, int64_t);                                    \
  template void g_decomposition<T>(const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &,  \
                                   size_t, size_t);                                                              \
  template void ntt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,        \
                       const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,        \
                       const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,        \
                       std::shared_ptr<DeviceTensor<T>> &);                                                      \
  template void intt<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,       \
                        const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,       \
                        const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,       \
                        const std::shared_ptr<DeviceTensor<T>> &, std::shared_ptr<DeviceTensor<T>> &);           \
  template void permute<T>(const std::shared_ptr<DeviceTensor<T>> &, const std::shared_ptr<DeviceTensor<T>> &,    \
                           std::shared_ptr<DeviceTensor<T>> &, int64_t, int64_t);

HEAL_MEMORY(int32_t)
HEAL_MEMORY(int64_t)
HEAL_MEMORY(double)
HEAL_COMPUTE(int32_t)
HEAL_COMPUTE(int64_t)

}  // namespace lattica_hw_api
