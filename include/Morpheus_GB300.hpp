// Morpheus_GB300.hpp -- header-only C++17 front end of morpheus-gb300.
//
// Keeps the reference's template API for the SpMV hot path so that code
// written against Morpheus switches by changing the execution space:
//
//   Morpheus::CsrMatrix<double> A(...);                 // device containers
//   Morpheus::multiply<Morpheus::GB300>(A, x, y);       // core/src/Morpheus_Multiply.hpp:57-78
//   Morpheus::multiply<Morpheus::GB300>(A, x, y, false);// y += A*x
//   double d = Morpheus::dot<Morpheus::GB300>(n, x, y); // core/src/Morpheus_Dot.hpp:50-58
//   double s = Morpheus::reduce<Morpheus::GB300>(x, n); // core/src/Morpheus_Reduction.hpp:46-52
//   Morpheus::waxpby<Morpheus::GB300>(n, a, x, b, y, w);// core/src/Morpheus_WAXPBY.hpp:52-64
//   Morpheus::convert<Morpheus::GB300>(src, dst);       // core/src/Morpheus_Convert.hpp:53-57
//   Morpheus::convert<Morpheus::GB300>(dyn, fmt);       // core/src/Morpheus_Convert.hpp:88-141
//
// Containers own device memory (RAII over cudaMalloc) and expose the
// reference's accessors (nrows(), ncols(), nnnz(), row_offsets(), ...).
// Every algorithm calls the C ABI of mgb.h; a non-success status is rethrown
// as the reference's exception class (core/src/Morpheus_Exceptions.hpp:32-73).
#ifndef MORPHEUS_GB300_HPP
#define MORPHEUS_GB300_HPP

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <variant>
#include <vector>

#include "mgb.h"

namespace Morpheus {

// ---------------------------------------------------------------- spaces ---
// The GB300 execution space: algorithms templated on it run the sm_103a
// kernels of libmorpheus_gb300.so on the current CUDA device.
struct GB300 {
  using execution_space = GB300;
};

// ----------------------------------------------------------- exceptions ---
class Exception : public std::exception {
 public:
  explicit Exception(std::string m) : message(std::move(m)) {}
  const char* what() const noexcept override { return message.c_str(); }

 protected:
  std::string message;
};
class NotImplementedException : public Exception {
 public:
  explicit NotImplementedException(const std::string& fn)
      : Exception("NotImplemented: " + fn + " not yet implemented.") {}
};
class IOException : public Exception {
 public:
  explicit IOException(const std::string& m) : Exception("IO: " + m) {}
};
class RuntimeException : public Exception {
 public:
  explicit RuntimeException(const std::string& m) : Exception(m) {}
};
class InvalidInputException : public Exception {
 public:
  explicit InvalidInputException(const std::string& m) : Exception(m) {}
};
class FormatConversionException : public Exception {
 public:
  explicit FormatConversionException(const std::string& m) : Exception(m) {}
};

namespace Impl {
inline void check(int st, const char* where) {
  if (st == MGB_SUCCESS) return;
  std::string msg = std::string(where) + ": " + mgb_status_string(st);
  if (st == MGB_ERR_CUDA || st == MGB_ERR_ALLOC) msg += std::string(" (") + mgb_last_cuda_error_string() + ")";
  switch (st) {
    case MGB_ERR_NOT_IMPLEMENTED: throw NotImplementedException(where);
    case MGB_ERR_FORMAT_CONVERSION: throw FormatConversionException(msg);
    case MGB_ERR_INVALID_INPUT:
    case MGB_ERR_BAD_ARGUMENT: throw InvalidInputException(msg);
    case MGB_ERR_IO: throw IOException(msg);
    default: throw RuntimeException(msg);
  }
}
inline void cuda_check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw RuntimeException(std::string(where) + ": " + cudaGetErrorString(e));
}
inline int64_t get_pad_size(int64_t len, int64_t alignment) {  // impl/Dia/Morpheus_Utils_Impl.hpp:33-36
  return alignment * ((len + alignment - 1) / alignment);
}
}  // namespace Impl

// ------------------------------------------------------------- enums ---
enum formats_e { COO_FORMAT = 0, CSR_FORMAT, DIA_FORMAT, ELL_FORMAT, HYB_FORMAT, HDC_FORMAT, NFORMATS };
enum conversion_error_e { DYNAMIC_TO_PROXY = 0, PROXY_TO_DYNAMIC, CONV_SUCCESS };

// ------------------------------------------------------- device buffer ---
template <class T>
class DeviceArray {
 public:
  DeviceArray() = default;
  explicit DeviceArray(size_t n, T fill = T(0)) { resize(n, fill); }
  explicit DeviceArray(const std::vector<T>& host) { assign(host); }
  DeviceArray(const DeviceArray& o) { *this = o; }
  DeviceArray(DeviceArray&& o) noexcept : ptr_(o.ptr_), n_(o.n_) { o.ptr_ = nullptr; o.n_ = 0; }
  DeviceArray& operator=(const DeviceArray& o) {  // deep copy (device to device)
    if (this != &o) {
      alloc(o.n_);
      if (n_) Impl::cuda_check(cudaMemcpy(ptr_, o.ptr_, n_ * sizeof(T), cudaMemcpyDeviceToDevice), "copy");
    }
    return *this;
  }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    std::swap(ptr_, o.ptr_);
    std::swap(n_, o.n_);
    return *this;
  }
  ~DeviceArray() { release(); }

  void resize(size_t n, T fill = T(0)) {
    alloc(n);
    if (n_) assign_fill(fill);
  }
  void assign(const std::vector<T>& host) {
    alloc(host.size());
    if (n_) Impl::cuda_check(cudaMemcpy(ptr_, host.data(), n_ * sizeof(T), cudaMemcpyHostToDevice), "upload");
  }
  std::vector<T> to_host() const {
    std::vector<T> h(n_);
    if (n_) Impl::cuda_check(cudaMemcpy(h.data(), ptr_, n_ * sizeof(T), cudaMemcpyDeviceToHost), "download");
    return h;
  }
  T* data() { return ptr_; }
  const T* data() const { return ptr_; }
  size_t size() const { return n_; }

 private:
  void alloc(size_t n) {
    if (n == n_) return;
    release();
    if (n) Impl::cuda_check(cudaMalloc((void**)&ptr_, n * sizeof(T)), "cudaMalloc");
    n_ = n;
  }
  void release() {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    n_ = 0;
  }
  void assign_fill(T fill) {
    if (fill == T(0)) {
      Impl::cuda_check(cudaMemset(ptr_, 0, n_ * sizeof(T)), "memset");
    } else {
      std::vector<T> h(n_, fill);
      Impl::cuda_check(cudaMemcpy(ptr_, h.data(), n_ * sizeof(T), cudaMemcpyHostToDevice), "fill");
    }
  }
  T* ptr_ = nullptr;
  size_t n_ = 0;
};

// ---------------------------------------------------------- DenseVector ---
// core/src/Morpheus_DenseVector.hpp (device space)
template <class ValueType>
class DenseVector {
 public:
  using value_type = ValueType;
  DenseVector() = default;
  explicit DenseVector(size_t n, ValueType v = ValueType(0)) : a_(n, v) {}
  explicit DenseVector(const std::vector<ValueType>& h) : a_(h) {}
  size_t size() const { return a_.size(); }
  ValueType* data() { return a_.data(); }
  const ValueType* data() const { return a_.data(); }
  void assign(size_t n, ValueType v) { a_.resize(n, v); }
  std::vector<ValueType> to_host() const { return a_.to_host(); }

 private:
  DeviceArray<ValueType> a_;
};

// ------------------------------------------------------------ matrices ---
template <class ValueType>
class CooMatrix {  // core/src/Morpheus_CooMatrix.hpp
 public:
  using value_type = ValueType;
  static constexpr formats_e format = COO_FORMAT;
  CooMatrix() = default;
  CooMatrix(int64_t r, int64_t c, int64_t n) { resize(r, c, n); }
  CooMatrix(int64_t r, int64_t c, const std::vector<int32_t>& ri, const std::vector<int32_t>& ci,
            const std::vector<ValueType>& v)
      : nrows_(r), ncols_(c), nnz_((int64_t)v.size()), ri_(ri), ci_(ci), v_(v) {}
  void resize(int64_t r, int64_t c, int64_t n) {
    nrows_ = r; ncols_ = c; nnz_ = n;
    ri_.resize(n); ci_.resize(n); v_.resize(n);
  }
  int64_t nrows() const { return nrows_; }
  int64_t ncols() const { return ncols_; }
  int64_t nnnz() const { return nnz_; }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  DeviceArray<int32_t>& row_indices() { return ri_; }
  DeviceArray<int32_t>& column_indices() { return ci_; }
  DeviceArray<ValueType>& values() { return v_; }
  const DeviceArray<int32_t>& crow_indices() const { return ri_; }
  const DeviceArray<int32_t>& ccolumn_indices() const { return ci_; }
  const DeviceArray<ValueType>& cvalues() const { return v_; }
  mgb_coo desc() const {
    return mgb_coo{nrows_, ncols_, nnz_, const_cast<int32_t*>(ri_.data()), const_cast<int32_t*>(ci_.data()),
                   const_cast<ValueType*>(v_.data())};
  }

 private:
  int64_t nrows_ = 0, ncols_ = 0, nnz_ = 0;
  DeviceArray<int32_t> ri_, ci_;
  DeviceArray<ValueType> v_;
};

template <class ValueType>
class CsrMatrix {  // core/src/Morpheus_CsrMatrix.hpp:533-537
 public:
  using value_type = ValueType;
  static constexpr formats_e format = CSR_FORMAT;
  CsrMatrix() = default;
  CsrMatrix(int64_t r, int64_t c, int64_t n) { resize(r, c, n); }
  CsrMatrix(int64_t r, int64_t c, const std::vector<int32_t>& ro, const std::vector<int32_t>& ci,
            const std::vector<ValueType>& v)
      : nrows_(r), ncols_(c), nnz_((int64_t)v.size()), ro_(ro), ci_(ci), v_(v) {}
  void resize(int64_t r, int64_t c, int64_t n) {
    nrows_ = r; ncols_ = c; nnz_ = n;
    ro_.resize(r + 1); ci_.resize(n); v_.resize(n);
    forget_kernel_variant();
  }
  // SpMV kernel of this matrix (MGB_CSR_ROWS, MGB_CSR_SEGMENTS or
  // MGB_CSR_SPLIT), measured on the device at the first multiply and cached,
  // and for the lane-segment kernel its chunk plan (mgb_csr_plan).  Both
  // depend on the row offsets only: the non-const row_offsets() accessor and
  // resize() drop them; call forget_kernel_variant() after writing new row
  // offsets through a pointer kept from earlier.
  int kernel_variant() const;
  const int32_t* chunk_plan(int64_t* entries) const;
  void forget_kernel_variant() {
    variant_ = 0;
    plan_ok_ = false;
  }
  int64_t nrows() const { return nrows_; }
  int64_t ncols() const { return ncols_; }
  int64_t nnnz() const { return nnz_; }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  DeviceArray<int32_t>& row_offsets() {
    forget_kernel_variant();
    return ro_;
  }
  DeviceArray<int32_t>& column_indices() { return ci_; }
  DeviceArray<ValueType>& values() { return v_; }
  const DeviceArray<int32_t>& crow_offsets() const { return ro_; }
  const DeviceArray<int32_t>& ccolumn_indices() const { return ci_; }
  const DeviceArray<ValueType>& cvalues() const { return v_; }
  mgb_csr desc() const {
    return mgb_csr{nrows_, ncols_, nnz_, const_cast<int32_t*>(ro_.data()), const_cast<int32_t*>(ci_.data()),
                   const_cast<ValueType*>(v_.data())};
  }

 private:
  int64_t nrows_ = 0, ncols_ = 0, nnz_ = 0;
  DeviceArray<int32_t> ro_, ci_;
  DeviceArray<ValueType> v_;
  mutable int variant_ = 0;
  mutable DeviceArray<int32_t> plan_;
  mutable bool plan_ok_ = false;
};

template <class ValueType>
int CsrMatrix<ValueType>::kernel_variant() const {
  if (variant_ == 0) {
    mgb_csr d = desc();
    int v = MGB_CSR_SEGMENTS;
    Impl::check(mgb_csr_choose_kernel(&d, &v, nullptr), "CsrMatrix::kernel_variant");
    variant_ = v;
  }
  return variant_;
}

template <class ValueType>
const int32_t* CsrMatrix<ValueType>::chunk_plan(int64_t* entries) const {
  mgb_csr d = desc();
  int64_t n = 0;
  Impl::check(mgb_csr_plan_entries(&d, &n), "CsrMatrix::chunk_plan");
  if (!plan_ok_ || (int64_t)plan_.size() != n) {
    plan_.resize((size_t)n);
    Impl::check(mgb_csr_plan(&d, plan_.data(), n, nullptr), "CsrMatrix::chunk_plan");
    plan_ok_ = true;
  }
  *entries = n;
  return plan_.data();
}

template <class ValueType>
class DiaMatrix {  // core/src/Morpheus_DiaMatrix.hpp:192-201, values (pad(N,32) x ndiags) column-major
 public:
  using value_type = ValueType;
  static constexpr formats_e format = DIA_FORMAT;
  DiaMatrix() = default;
  DiaMatrix(int64_t r, int64_t c, int64_t n, int64_t nd, int64_t align = 32) { resize(r, c, n, nd, align); }
  DiaMatrix(int64_t r, int64_t c, int64_t n, const std::vector<int32_t>& offs,
            const std::vector<ValueType>& vals, int64_t align = 32)
      : nrows_(r), ncols_(c), nnz_(n), ndiags_((int64_t)offs.size()), align_(align),
        pitch_(Impl::get_pad_size(r, align)), off_(offs), v_(vals) {
    if ((int64_t)vals.size() != pitch_ * ndiags_) throw InvalidInputException("DIA values size");
  }
  void resize(int64_t r, int64_t c, int64_t n, int64_t nd, int64_t align = 32) {
    nrows_ = r; ncols_ = c; nnz_ = n; ndiags_ = nd; align_ = align;
    pitch_ = Impl::get_pad_size(r, align);
    off_.resize(nd); v_.resize(pitch_ * nd);
  }
  int64_t nrows() const { return nrows_; }
  int64_t ncols() const { return ncols_; }
  int64_t nnnz() const { return nnz_; }
  int64_t ndiags() const { return ndiags_; }
  int64_t alignment() const { return align_; }
  int64_t pitch() const { return pitch_; }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  DeviceArray<int32_t>& diagonal_offsets() { return off_; }
  DeviceArray<ValueType>& values() { return v_; }
  const DeviceArray<int32_t>& cdiagonal_offsets() const { return off_; }
  const DeviceArray<ValueType>& cvalues() const { return v_; }
  mgb_dia desc() const {
    return mgb_dia{nrows_, ncols_, nnz_, ndiags_, pitch_, const_cast<int32_t*>(off_.data()),
                   const_cast<ValueType*>(v_.data())};
  }

 private:
  int64_t nrows_ = 0, ncols_ = 0, nnz_ = 0, ndiags_ = 0, align_ = 32, pitch_ = 0;
  DeviceArray<int32_t> off_;
  DeviceArray<ValueType> v_;
};

template <class ValueType>
class EllMatrix {  // core/src/Morpheus_EllMatrix.hpp:189-202; slots (N x pad(W,32)) column-major
 public:
  using value_type = ValueType;
  static constexpr formats_e format = ELL_FORMAT;
  static constexpr int32_t invalid_index() { return MGB_INVALID_INDEX; }
  EllMatrix() = default;
  EllMatrix(int64_t r, int64_t c, int64_t n, int64_t epr, int64_t align = 32) { resize(r, c, n, epr, align); }
  EllMatrix(int64_t r, int64_t c, int64_t n, int64_t epr, const std::vector<int32_t>& ci,
            const std::vector<ValueType>& v, int64_t align = 32)
      : nrows_(r), ncols_(c), nnz_(n), epr_(epr), align_(align), width_(Impl::get_pad_size(epr, align)),
        ci_(ci), v_(v) {
    if ((int64_t)ci.size() != r * width_ || ci.size() != v.size()) throw InvalidInputException("ELL sizes");
  }
  void resize(int64_t r, int64_t c, int64_t n, int64_t epr, int64_t align = 32) {
    nrows_ = r; ncols_ = c; nnz_ = n; epr_ = epr; align_ = align;
    width_ = Impl::get_pad_size(epr, align);
    ci_.resize(r * width_, MGB_INVALID_INDEX);
    v_.resize(r * width_);
  }
  int64_t nrows() const { return nrows_; }
  int64_t ncols() const { return ncols_; }
  int64_t nnnz() const { return nnz_; }
  int64_t entries_per_row() const { return epr_; }
  int64_t alignment() const { return align_; }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  DeviceArray<int32_t>& column_indices() { return ci_; }
  DeviceArray<ValueType>& values() { return v_; }
  const DeviceArray<int32_t>& ccolumn_indices() const { return ci_; }
  const DeviceArray<ValueType>& cvalues() const { return v_; }
  mgb_ell desc() const {
    return mgb_ell{nrows_, ncols_, nnz_, epr_, width_, nrows_, const_cast<int32_t*>(ci_.data()),
                   const_cast<ValueType*>(v_.data())};
  }

 private:
  int64_t nrows_ = 0, ncols_ = 0, nnz_ = 0, epr_ = 0, align_ = 32, width_ = 0;
  DeviceArray<int32_t> ci_;
  DeviceArray<ValueType> v_;
};

template <class ValueType>
class HybMatrix {  // core/src/Morpheus_HybMatrix.hpp:473-476
 public:
  using value_type = ValueType;
  static constexpr formats_e format = HYB_FORMAT;
  HybMatrix() = default;
  HybMatrix(EllMatrix<ValueType> e, CooMatrix<ValueType> c) : ell_(std::move(e)), coo_(std::move(c)) {}
  int64_t nrows() const { return ell_.nrows(); }
  int64_t ncols() const { return ell_.ncols(); }
  int64_t nnnz() const { return ell_.nnnz() + coo_.nnnz(); }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  EllMatrix<ValueType>& ell() { return ell_; }
  CooMatrix<ValueType>& coo() { return coo_; }
  const EllMatrix<ValueType>& cell() const { return ell_; }
  const CooMatrix<ValueType>& ccoo() const { return coo_; }
  mgb_hyb desc() const { return mgb_hyb{ell_.desc(), coo_.desc()}; }

 private:
  EllMatrix<ValueType> ell_;
  CooMatrix<ValueType> coo_;
};

template <class ValueType>
class HdcMatrix {  // core/src/Morpheus_HdcMatrix.hpp:464-467
 public:
  using value_type = ValueType;
  static constexpr formats_e format = HDC_FORMAT;
  static constexpr double true_diagonal_ratio = 0.2;
  HdcMatrix() = default;
  HdcMatrix(DiaMatrix<ValueType> d, CsrMatrix<ValueType> c) : dia_(std::move(d)), csr_(std::move(c)) {}
  int64_t nrows() const { return dia_.nrows(); }
  int64_t ncols() const { return dia_.ncols(); }
  int64_t nnnz() const { return dia_.nnnz() + csr_.nnnz(); }
  formats_e format_enum() const { return format; }
  int format_index() const { return format; }
  DiaMatrix<ValueType>& dia() { return dia_; }
  CsrMatrix<ValueType>& csr() { return csr_; }
  const DiaMatrix<ValueType>& cdia() const { return dia_; }
  const CsrMatrix<ValueType>& ccsr() const { return csr_; }
  mgb_hdc desc() const { return mgb_hdc{dia_.desc(), csr_.desc()}; }

 private:
  DiaMatrix<ValueType> dia_;
  CsrMatrix<ValueType> csr_;
};

// ---------------------------------------------------------- DynamicMatrix ---
// core/src/Morpheus_DynamicMatrix.hpp:102-462
template <class ValueType>
class DynamicMatrix {
 public:
  using value_type = ValueType;
  using variant_type = std::variant<CooMatrix<ValueType>, CsrMatrix<ValueType>, DiaMatrix<ValueType>,
                                    EllMatrix<ValueType>, HybMatrix<ValueType>, HdcMatrix<ValueType>>;
  DynamicMatrix() = default;
  DynamicMatrix(const DynamicMatrix&) = default;
  DynamicMatrix(DynamicMatrix&&) noexcept = default;
  DynamicMatrix& operator=(const DynamicMatrix&) = default;
  DynamicMatrix& operator=(DynamicMatrix&&) noexcept = default;
  template <class M, class = std::enable_if_t<!std::is_same_v<std::decay_t<M>, DynamicMatrix>>>
  DynamicMatrix(M m) : v_(std::move(m)) {}
  template <class M, class = std::enable_if_t<!std::is_same_v<std::decay_t<M>, DynamicMatrix>>>
  DynamicMatrix& operator=(M m) {
    v_ = std::move(m);
    return *this;
  }
  int active_index() const { return (int)v_.index(); }
  formats_e active_enum() const { return (formats_e)v_.index(); }
  // Switches to an EMPTY container of the new format (no data is converted);
  // the active format, or an index past the last format, leaves the matrix
  // unchanged (core/src/Morpheus_DynamicMatrix.hpp:409-442).
  void activate(int idx) {
    if (idx == active_index()) return;
    switch (idx) {
      case COO_FORMAT: v_ = CooMatrix<ValueType>(); break;
      case CSR_FORMAT: v_ = CsrMatrix<ValueType>(); break;
      case DIA_FORMAT: v_ = DiaMatrix<ValueType>(); break;
      case ELL_FORMAT: v_ = EllMatrix<ValueType>(); break;
      case HYB_FORMAT: v_ = HybMatrix<ValueType>(); break;
      case HDC_FORMAT: v_ = HdcMatrix<ValueType>(); break;
      default: break;
    }
  }
  void activate(formats_e f) { activate((int)f); }
  int64_t nrows() const { return std::visit([](const auto& m) { return m.nrows(); }, v_); }
  int64_t ncols() const { return std::visit([](const auto& m) { return m.ncols(); }, v_); }
  int64_t nnnz() const { return std::visit([](const auto& m) { return m.nnnz(); }, v_); }
  variant_type& formats() { return v_; }
  const variant_type& const_formats() const { return v_; }

 private:
  variant_type v_;
};

// ----------------------------------------------------------- algorithms ---
namespace Impl {
template <class ExecSpace>
constexpr void require_gb300() {
  static_assert(std::is_same_v<typename ExecSpace::execution_space, GB300>,
                "Morpheus_GB300.hpp implements the GB300 execution space only");
}
template <class T> struct Suffix;
template <> struct Suffix<double> {
  static int csr(const mgb_csr* a, const double* x, double* y, int i, int v, void* s) {
    return mgb_spmv_csr_variant_f64(a, x, y, i, v, s);
  }
  static int csr_planned(const mgb_csr* a, const int32_t* p, int64_t n, const double* x, double* y, int i, void* s) {
    return mgb_spmv_csr_planned_f64(a, p, n, x, y, i, s);
  }
  static int coo(const mgb_coo* a, const double* x, double* y, int i, void* s) { return mgb_spmv_coo_f64(a, x, y, i, s); }
  static int dia(const mgb_dia* a, const double* x, double* y, int i, void* s) { return mgb_spmv_dia_f64(a, x, y, i, s); }
  static int ell(const mgb_ell* a, const double* x, double* y, int i, void* s) { return mgb_spmv_ell_f64(a, x, y, i, s); }
  static int hyb(const mgb_hyb* a, const double* x, double* y, int i, void* s) { return mgb_spmv_hyb_f64(a, x, y, i, s); }
  static int hdc(const mgb_hdc* a, const double* x, double* y, int i, void* s) { return mgb_spmv_hdc_f64(a, x, y, i, s); }
  static int dot(int64_t n, const double* x, const double* y, double* r) { return mgb_dot_f64(n, x, y, r, nullptr); }
  static int reduce(const double* x, int64_t n, double* r) { return mgb_reduce_f64(x, n, r, nullptr); }
  static int waxpby(int64_t n, double a, const double* x, double b, const double* y, double* w) {
    return mgb_waxpby_f64(n, a, x, b, y, w, nullptr);
  }
};
template <> struct Suffix<float> {
  static int csr(const mgb_csr* a, const float* x, float* y, int i, int v, void* s) {
    return mgb_spmv_csr_variant_f32(a, x, y, i, v, s);
  }
  static int csr_planned(const mgb_csr* a, const int32_t* p, int64_t n, const float* x, float* y, int i, void* s) {
    return mgb_spmv_csr_planned_f32(a, p, n, x, y, i, s);
  }
  static int coo(const mgb_coo* a, const float* x, float* y, int i, void* s) { return mgb_spmv_coo_f32(a, x, y, i, s); }
  static int dia(const mgb_dia* a, const float* x, float* y, int i, void* s) { return mgb_spmv_dia_f32(a, x, y, i, s); }
  static int ell(const mgb_ell* a, const float* x, float* y, int i, void* s) { return mgb_spmv_ell_f32(a, x, y, i, s); }
  static int hyb(const mgb_hyb* a, const float* x, float* y, int i, void* s) { return mgb_spmv_hyb_f32(a, x, y, i, s); }
  static int hdc(const mgb_hdc* a, const float* x, float* y, int i, void* s) { return mgb_spmv_hdc_f32(a, x, y, i, s); }
  static int dot(int64_t n, const float* x, const float* y, float* r) { return mgb_dot_f32(n, x, y, r, nullptr); }
  static int reduce(const float* x, int64_t n, float* r) { return mgb_reduce_f32(x, n, r, nullptr); }
  static int waxpby(int64_t n, float a, const float* x, float b, const float* y, float* w) {
    return mgb_waxpby_f32(n, a, x, b, y, w, nullptr);
  }
};

template <class T>
void spmv(const CsrMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  const int v = A.kernel_variant();
  if (v == MGB_CSR_SEGMENTS) {
    int64_t n = 0;
    const int32_t* plan = A.chunk_plan(&n);
    check(Suffix<T>::csr_planned(&d, plan, n, x, y, init, nullptr), "multiply<GB300>(CsrMatrix)");
  } else {
    check(Suffix<T>::csr(&d, x, y, init, v, nullptr), "multiply<GB300>(CsrMatrix)");
  }
}
template <class T>
void spmv(const CooMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  check(Suffix<T>::coo(&d, x, y, init, nullptr), "multiply<GB300>(CooMatrix)");
}
template <class T>
void spmv(const DiaMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  check(Suffix<T>::dia(&d, x, y, init, nullptr), "multiply<GB300>(DiaMatrix)");
}
template <class T>
void spmv(const EllMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  check(Suffix<T>::ell(&d, x, y, init, nullptr), "multiply<GB300>(EllMatrix)");
}
template <class T>
void spmv(const HybMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  check(Suffix<T>::hyb(&d, x, y, init, nullptr), "multiply<GB300>(HybMatrix)");
}
template <class T>
void spmv(const HdcMatrix<T>& A, const T* x, T* y, bool init) {
  auto d = A.desc();
  check(Suffix<T>::hdc(&d, x, y, init, nullptr), "multiply<GB300>(HdcMatrix)");
}
template <class T>
void spmv(const DynamicMatrix<T>& A, const T* x, T* y, bool init) {  // impl/Dynamic/Morpheus_Multiply_Impl.hpp:35-44
  std::visit([&](const auto& m) { spmv(m, x, y, init); }, A.const_formats());
}
}  // namespace Impl

// core/src/Morpheus_Multiply.hpp:57-61
template <class ExecSpace, class Matrix, class Vector>
inline void multiply(const Matrix& A, const Vector& x, Vector& y, const bool init) {
  Impl::require_gb300<ExecSpace>();
  if ((int64_t)x.size() < A.ncols() || (int64_t)y.size() < A.nrows())
    throw InvalidInputException("multiply: vector sizes do not match the matrix");
  Impl::spmv(A, x.data(), y.data(), init);
}

// core/src/Morpheus_Multiply.hpp:75-78
template <class ExecSpace, class Matrix, class Vector>
inline void multiply(const Matrix& A, const Vector& x, Vector& y) {
  multiply<ExecSpace>(A, x, y, true);
}

// core/src/Morpheus_Dot.hpp:50-58
template <class ExecSpace, class Vector1, class Vector2>
inline typename Vector2::value_type dot(size_t n, const Vector1& x, const Vector2& y) {
  Impl::require_gb300<ExecSpace>();
  typename Vector2::value_type r{};
  Impl::check(Impl::Suffix<typename Vector2::value_type>::dot((int64_t)n, x.data(), y.data(), &r), "dot<GB300>");
  return r;
}

// core/src/Morpheus_Reduction.hpp:46-52
template <class ExecSpace, class Vector>
inline typename Vector::value_type reduce(const Vector& in, size_t size) {
  Impl::require_gb300<ExecSpace>();
  typename Vector::value_type r{};
  Impl::check(Impl::Suffix<typename Vector::value_type>::reduce(in.data(), (int64_t)size, &r), "reduce<GB300>");
  return r;
}

// core/src/Morpheus_WAXPBY.hpp:52-64
template <class ExecSpace, class Vector1, class Vector2, class Vector3>
inline void waxpby(size_t n, typename Vector1::value_type alpha, const Vector1& x,
                   typename Vector2::value_type beta, const Vector2& y, Vector3& w) {
  Impl::require_gb300<ExecSpace>();
  Impl::check(Impl::Suffix<typename Vector1::value_type>::waxpby((int64_t)n, alpha, x.data(), beta, y.data(),
                                                                 w.data()),
              "waxpby<GB300>");
}

// -------------------------------------------------------------- convert ---
// Every pair goes through COO on the device (impl/Morpheus_Convert_Impl.hpp:82-104);
// the structures are bit-identical to the reference's Serial convert.
namespace Impl {
template <class T> struct Conv;
#define MGB_CONV_ENTRIES(SFX)                                                                                      \
  static int csr_to_coo(const mgb_csr* s, mgb_coo* d) { return mgb_convert_csr_to_coo_##SFX(s, d, nullptr); }    \
  static int coo_to_csr(const mgb_coo* s, mgb_csr* d) { return mgb_convert_coo_to_csr_##SFX(s, d, nullptr); }    \
  static int dia_to_coo(const mgb_dia* s, mgb_coo* d) { return mgb_convert_dia_to_coo_##SFX(s, d, nullptr); }    \
  static int coo_to_dia(const mgb_coo* s, mgb_dia* d) { return mgb_convert_coo_to_dia_##SFX(s, d, nullptr); }    \
  static int ell_to_coo(const mgb_ell* s, mgb_coo* d) { return mgb_convert_ell_to_coo_##SFX(s, d, nullptr); }    \
  static int coo_to_ell(const mgb_coo* s, mgb_ell* d) { return mgb_convert_coo_to_ell_##SFX(s, d, nullptr); }    \
  static int hyb_to_coo(const mgb_hyb* s, mgb_coo* d) { return mgb_convert_hyb_to_coo_##SFX(s, d, nullptr); }    \
  static int coo_to_hyb(const mgb_coo* s, mgb_hyb* d) { return mgb_convert_coo_to_hyb_##SFX(s, d, nullptr); }    \
  static int hdc_to_coo(const mgb_hdc* s, mgb_coo* d) { return mgb_convert_hdc_to_coo_##SFX(s, d, nullptr); }    \
  static int coo_to_hdc(const mgb_coo* s, mgb_hdc* d) { return mgb_convert_coo_to_hdc_##SFX(s, d, nullptr); }    \
  static int sort(mgb_coo* a) { return mgb_coo_sort_by_row_and_column_##SFX(a, nullptr); }
template <> struct Conv<double> { MGB_CONV_ENTRIES(f64) };
template <> struct Conv<float> { MGB_CONV_ENTRIES(f32) };
#undef MGB_CONV_ENTRIES

// X -> COO
template <class T>
CooMatrix<T> to_coo(const CooMatrix<T>& A) { return A; }
template <class T>
CooMatrix<T> to_coo(const CsrMatrix<T>& A) {
  CooMatrix<T> out(A.nrows(), A.ncols(), A.nnnz());
  mgb_csr s = A.desc();
  mgb_coo d = out.desc();
  check(Conv<T>::csr_to_coo(&s, &d), "convert<GB300>(CsrMatrix -> CooMatrix)");
  return out;
}
template <class T>
CooMatrix<T> to_coo(const DiaMatrix<T>& A) {
  CooMatrix<T> out(A.nrows(), A.ncols(), A.nnnz());
  mgb_dia s = A.desc();
  mgb_coo d = out.desc();
  check(Conv<T>::dia_to_coo(&s, &d), "convert<GB300>(DiaMatrix -> CooMatrix)");
  return out;
}
template <class T>
CooMatrix<T> to_coo(const EllMatrix<T>& A) {
  CooMatrix<T> out(A.nrows(), A.ncols(), A.nnnz());
  mgb_ell s = A.desc();
  mgb_coo d = out.desc();
  check(Conv<T>::ell_to_coo(&s, &d), "convert<GB300>(EllMatrix -> CooMatrix)");
  return out;
}
template <class T>
CooMatrix<T> to_coo(const HybMatrix<T>& A) {
  CooMatrix<T> out(A.nrows(), A.ncols(), A.nnnz());
  mgb_hyb s = A.desc();
  mgb_coo d = out.desc();
  check(Conv<T>::hyb_to_coo(&s, &d), "convert<GB300>(HybMatrix -> CooMatrix)");
  return out;
}
template <class T>
CooMatrix<T> to_coo(const HdcMatrix<T>& A) {
  CooMatrix<T> out(A.nrows(), A.ncols(), A.nnnz());
  mgb_hdc s = A.desc();
  mgb_coo d = out.desc();
  check(Conv<T>::hdc_to_coo(&s, &d), "convert<GB300>(HdcMatrix -> CooMatrix)");
  return out;
}
template <class T>
CooMatrix<T> to_coo(const DynamicMatrix<T>& A) {
  return std::visit([](const auto& m) { return to_coo(m); }, A.const_formats());
}

// COO -> Y (sizes from the *_plan calls, which also apply the fill tolerance)
template <class T>
void from_coo(const CooMatrix<T>& A, CooMatrix<T>& out) { out = A; }
template <class T>
void from_coo(const CooMatrix<T>& A, CsrMatrix<T>& out) {
  mgb_coo s = A.desc();
  CsrMatrix<T> r(A.nrows(), A.ncols(), A.nnnz());
  mgb_csr d = r.desc();
  check(Conv<T>::coo_to_csr(&s, &d), "convert<GB300>(CooMatrix -> CsrMatrix)");
  out = std::move(r);
}
template <class T>
void from_coo(const CooMatrix<T>& A, DiaMatrix<T>& out) {
  mgb_coo s = A.desc();
  int64_t nd = 0;
  check(mgb_convert_coo_to_dia_plan(&s, &nd, nullptr), "convert<GB300>(CooMatrix -> DiaMatrix)");
  DiaMatrix<T> r(A.nrows(), A.ncols(), A.nnnz(), nd);
  mgb_dia d = r.desc();
  check(Conv<T>::coo_to_dia(&s, &d), "convert<GB300>(CooMatrix -> DiaMatrix)");
  out = std::move(r);
}
template <class T>
void from_coo(const CooMatrix<T>& A, EllMatrix<T>& out) {
  mgb_coo s = A.desc();
  int64_t w = 0;
  check(mgb_convert_coo_to_ell_plan(&s, &w, nullptr), "convert<GB300>(CooMatrix -> EllMatrix)");
  EllMatrix<T> r(A.nrows(), A.ncols(), A.nnnz(), w);
  mgb_ell d = r.desc();
  check(Conv<T>::coo_to_ell(&s, &d), "convert<GB300>(CooMatrix -> EllMatrix)");
  out = std::move(r);
}
template <class T>
void from_coo(const CooMatrix<T>& A, HybMatrix<T>& out) {
  mgb_coo s = A.desc();
  int64_t w = 0, ell_nnz = 0, coo_nnz = 0;
  check(mgb_convert_coo_to_hyb_plan(&s, 0, &w, &ell_nnz, &coo_nnz, nullptr), "convert<GB300>(CooMatrix -> HybMatrix)");
  HybMatrix<T> r(EllMatrix<T>(A.nrows(), A.ncols(), ell_nnz, w), CooMatrix<T>(A.nrows(), A.ncols(), coo_nnz));
  mgb_hyb d = r.desc();
  check(Conv<T>::coo_to_hyb(&s, &d), "convert<GB300>(CooMatrix -> HybMatrix)");
  out = std::move(r);
}
template <class T>
void from_coo(const CooMatrix<T>& A, HdcMatrix<T>& out) {
  mgb_coo s = A.desc();
  int64_t nd = 0, dia_nnz = 0, csr_nnz = 0;
  check(mgb_convert_coo_to_hdc_plan(&s, &nd, &dia_nnz, &csr_nnz, nullptr), "convert<GB300>(CooMatrix -> HdcMatrix)");
  HdcMatrix<T> r(DiaMatrix<T>(A.nrows(), A.ncols(), dia_nnz, nd), CsrMatrix<T>(A.nrows(), A.ncols(), csr_nnz));
  mgb_hdc d = r.desc();
  check(Conv<T>::coo_to_hdc(&s, &d), "convert<GB300>(CooMatrix -> HdcMatrix)");
  out = std::move(r);
}
template <class T>
void from_coo(const CooMatrix<T>& A, DynamicMatrix<T>& out) {  // keeps the active format of out
  std::visit([&](auto& m) { from_coo(A, m); }, out.formats());
}
}  // namespace Impl

// core/src/Morpheus_Convert.hpp:53-57: src and dst of any (possibly the same)
// formats, including DynamicMatrix on either side.
template <class ExecSpace, class SourceType, class DestinationType>
void convert(const SourceType& src, DestinationType& dst) {
  Impl::require_gb300<ExecSpace>();
  Impl::from_coo(Impl::to_coo(src), dst);
}

// core/src/Morpheus_Convert.hpp:88-124: in-place switch of a DynamicMatrix
// with the reference's error codes (the source is left unchanged on error).
template <class ExecSpace, class ValueType>
conversion_error_e convert(DynamicMatrix<ValueType>& A, const formats_e index) {
  Impl::require_gb300<ExecSpace>();
  const int idx = (int)index;
  if (idx < 0 || idx >= (int)NFORMATS) return PROXY_TO_DYNAMIC;
  if (A.active_index() == idx) return CONV_SUCCESS;
  CooMatrix<ValueType> temp;
  try {
    temp = Impl::to_coo(A);
  } catch (const Exception&) {
    return DYNAMIC_TO_PROXY;
  }
  DynamicMatrix<ValueType> out;
  out.activate(idx);
  try {
    Impl::from_coo(temp, out);
  } catch (const Exception&) {
    return PROXY_TO_DYNAMIC;
  }
  A = std::move(out);
  return CONV_SUCCESS;
}

// core/src/Morpheus_Convert.hpp:126-141
template <class ExecSpace, class ValueType>
conversion_error_e convert(DynamicMatrix<ValueType>& A, const int idx) {
  if (idx < 0 || idx >= (int)NFORMATS) return PROXY_TO_DYNAMIC;
  return convert<ExecSpace>(A, (formats_e)idx);
}

// impl/Coo/Serial/Morpheus_Sort_Impl.hpp:109-186
template <class ExecSpace, class ValueType>
void sort_by_row_and_column(CooMatrix<ValueType>& A) {
  Impl::require_gb300<ExecSpace>();
  mgb_coo d = A.desc();
  Impl::check(Impl::Conv<ValueType>::sort(&d), "sort_by_row_and_column<GB300>");
}
template <class ExecSpace, class ValueType>
bool is_sorted(const CooMatrix<ValueType>& A) {
  Impl::require_gb300<ExecSpace>();
  mgb_coo d = A.desc();
  int sorted = 0;
  Impl::check(mgb_coo_is_sorted(&d, &sorted, nullptr), "is_sorted<GB300>");
  return sorted != 0;
}

// ------------------------------------------------------------ analytics ---
// core/src/Morpheus_MatrixAnalytics.hpp:49-261 on the device, every format
// read in place with the reference's per-format counting rules (mgb.h).
namespace Impl {
// typed entry points (DIA / ELL / HYB / HDC per-diagonal counts read values;
// DIA / HDC features too)
template <class T> struct CountAbi;
#define MGB_COUNT_ENTRIES(sfx)                                                                                 \
  static int diag(const mgb_dia* a, int32_t* o, int i) { return mgb_count_nnz_per_diagonal_dia_##sfx(a, o, i, nullptr); } \
  static int diag(const mgb_ell* a, int32_t* o, int i) { return mgb_count_nnz_per_diagonal_ell_##sfx(a, o, i, nullptr); } \
  static int diag(const mgb_hyb* a, int32_t* o, int i) { return mgb_count_nnz_per_diagonal_hyb_##sfx(a, o, i, nullptr); } \
  static int diag(const mgb_hdc* a, int32_t* o, int i) { return mgb_count_nnz_per_diagonal_hdc_##sfx(a, o, i, nullptr); } \
  static int features(const mgb_dia* a, float* f, uint8_t* m) { return mgb_features_dia_##sfx(a, f, m, nullptr); }       \
  static int features(const mgb_hdc* a, float* f, uint8_t* m) { return mgb_features_hdc_##sfx(a, f, m, nullptr); }
template <> struct CountAbi<double> { MGB_COUNT_ENTRIES(f64) };
template <> struct CountAbi<float> { MGB_COUNT_ENTRIES(f32) };
#undef MGB_COUNT_ENTRIES
inline int features_of(const mgb_csr* a, float* f, uint8_t* m) { return mgb_features_csr(a, f, m, nullptr); }
inline int features_of(const mgb_coo* a, float* f, uint8_t* m) { return mgb_features_coo(a, f, m, nullptr); }
inline int features_of(const mgb_ell* a, float* f, uint8_t* m) { return mgb_features_ell(a, f, m, nullptr); }
inline int features_of(const mgb_hyb* a, float* f, uint8_t* m) { return mgb_features_hyb(a, f, m, nullptr); }
template <class T>
int features_of_typed(const mgb_dia* a, float* f, uint8_t* m) { return CountAbi<T>::features(a, f, m); }
template <class T>
int features_of_typed(const mgb_hdc* a, float* f, uint8_t* m) { return CountAbi<T>::features(a, f, m); }

template <class T>
void count_rows(const CsrMatrix<T>& A, int32_t* out, bool init) {
  mgb_csr d = A.desc();
  check(mgb_count_nnz_per_row_csr(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const CooMatrix<T>& A, int32_t* out, bool init) {
  mgb_coo d = A.desc();
  check(mgb_count_nnz_per_row_coo(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const DiaMatrix<T>& A, int32_t* out, bool init) {
  mgb_dia d = A.desc();
  check(mgb_count_nnz_per_row_dia(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const EllMatrix<T>& A, int32_t* out, bool init) {
  mgb_ell d = A.desc();
  check(mgb_count_nnz_per_row_ell(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const HybMatrix<T>& A, int32_t* out, bool init) {
  mgb_hyb d = A.desc();
  check(mgb_count_nnz_per_row_hyb(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const HdcMatrix<T>& A, int32_t* out, bool init) {
  mgb_hdc d = A.desc();
  check(mgb_count_nnz_per_row_hdc(&d, out, init, nullptr), "count_nnz_per_row<GB300>");
}
template <class T>
void count_rows(const DynamicMatrix<T>& A, int32_t* out, bool init) {
  std::visit([&](const auto& m) { count_rows(m, out, init); }, A.const_formats());
}
template <class T>
void count_diags(const CsrMatrix<T>& A, int32_t* out, bool init) {
  mgb_csr d = A.desc();
  check(mgb_count_nnz_per_diagonal_csr(&d, out, init, nullptr), "count_nnz_per_diagonal<GB300>");
}
template <class T>
void count_diags(const CooMatrix<T>& A, int32_t* out, bool init) {
  mgb_coo d = A.desc();
  check(mgb_count_nnz_per_diagonal_coo(&d, out, init, nullptr), "count_nnz_per_diagonal<GB300>");
}
template <class M>
void count_diags(const M& A, int32_t* out, bool init) {  // DIA, ELL, HYB, HDC
  const auto d = A.desc();
  check(CountAbi<typename M::value_type>::diag(&d, out, init), "count_nnz_per_diagonal<GB300>");
}
template <class T>
void count_diags(const DynamicMatrix<T>& A, int32_t* out, bool init) {
  std::visit([&](const auto& m) { count_diags(m, out, init); }, A.const_formats());
}
inline int64_t count_above(const DenseVector<int32_t>& v, int32_t threshold) {
  int64_t c = 0;
  check(mgb_count_nnz_vector(v.data(), (int64_t)v.size(), threshold, &c, nullptr), "count_nnz<GB300>");
  return c;
}
template <class Matrix>
std::vector<int32_t> row_lengths(const Matrix& A) {
  DenseVector<int32_t> v((size_t)A.nrows(), 0);
  count_rows(A, v.data(), true);
  return v.to_host();
}
}  // namespace Impl

template <class Matrix>
int64_t number_of_rows(const Matrix& A) { return A.nrows(); }
template <class Matrix>
int64_t number_of_columns(const Matrix& A) { return A.ncols(); }
template <class Matrix>
int64_t number_of_nnz(const Matrix& A) { return A.nnnz(); }
template <class Matrix>
double average_nnnz(const Matrix& A) { return (double)A.nnnz() / (double)A.nrows(); }
template <class Matrix>
double density(const Matrix& A) { return (double)A.nnnz() / ((double)A.nrows() * (double)A.ncols()); }

template <class ExecSpace, class Matrix>
void count_nnz_per_row(const Matrix& A, DenseVector<int32_t>& nnz_per_row, const bool init = true) {
  Impl::require_gb300<ExecSpace>();
  if ((int64_t)nnz_per_row.size() < A.nrows()) throw InvalidInputException("count_nnz_per_row: vector too short");
  Impl::count_rows(A, nnz_per_row.data(), init);
}

template <class ExecSpace, class Matrix>
void count_nnz_per_diagonal(const Matrix& A, DenseVector<int32_t>& nnz_per_diagonal, const bool init = true) {
  Impl::require_gb300<ExecSpace>();
  if ((int64_t)nnz_per_diagonal.size() < A.nrows() + A.ncols() - 1)
    throw InvalidInputException("count_nnz_per_diagonal: vector too short");
  Impl::count_diags(A, nnz_per_diagonal.data(), init);
}

// entries of a count vector that are > threshold and != 0
// (core/src/Morpheus_VectorAnalytics.hpp:124)
template <class ExecSpace>
int64_t count_nnz(const DenseVector<int32_t>& vec, int32_t threshold = 0) {
  Impl::require_gb300<ExecSpace>();
  return Impl::count_above(vec, threshold);
}

template <class ExecSpace, class Matrix>
int64_t max_nnnz(const Matrix& A) {
  Impl::require_gb300<ExecSpace>();
  int64_t m = 0;
  for (int32_t v : Impl::row_lengths(A)) m = v > m ? v : m;
  return m;
}

template <class ExecSpace, class Matrix>
int64_t min_nnnz(const Matrix& A) {
  Impl::require_gb300<ExecSpace>();
  const std::vector<int32_t> l = Impl::row_lengths(A);
  int64_t m = l.empty() ? 0 : l[0];
  for (int32_t v : l) m = v < m ? v : m;
  return m;
}

// Standard deviation of the row lengths about the true mean, as a double
// (the reference returns it truncated to an integer, about the integer mean
// nnz / nrows, core/src/Morpheus_MatrixAnalytics.hpp:177-193).
template <class ExecSpace, class Matrix>
double std_nnnz(const Matrix& A) {
  Impl::require_gb300<ExecSpace>();
  const std::vector<int32_t> l = Impl::row_lengths(A);
  if (l.empty()) return 0.0;
  const double mean = (double)A.nnnz() / (double)l.size();
  double acc = 0.0;
  for (int32_t v : l) acc += ((double)v - mean) * ((double)v - mean);
  return std::sqrt(acc / (double)l.size());
}

template <class ExecSpace, class Matrix>
int64_t count_diagonals(const Matrix& A) {
  Impl::require_gb300<ExecSpace>();
  DenseVector<int32_t> v((size_t)(A.nrows() + A.ncols() - 1), 0);
  Impl::count_diags(A, v.data(), true);
  return Impl::count_above(v, 0);
}

template <class ExecSpace, class Matrix>
int64_t count_true_diagonals(const Matrix& A, int32_t threshold) {
  Impl::require_gb300<ExecSpace>();
  DenseVector<int32_t> v((size_t)(A.nrows() + A.ncols() - 1), 0);
  Impl::count_diags(A, v.data(), true);
  return Impl::count_above(v, threshold);
}

// ------------------------------------------------------- solver steps ---
// Fused steps of an iterative solver and a device-resident CG (mgb.h, no
// reference counterpart).
namespace Impl {
template <class T> struct SolverAbi;
template <> struct SolverAbi<double> {
  static int spmv_dot(const mgb_csr* a, const double* x, double* y, int i, int v, double* d) {
    return mgb_spmv_dot_csr_f64(a, x, y, i, v, d, nullptr);
  }
  static int cg(const mgb_csr* a, int v, const double* b, double* x, int64_t m, double t, int64_t* it, double* r) {
    return mgb_cg_csr_f64(a, v, b, x, m, t, it, r, nullptr);
  }
};
template <> struct SolverAbi<float> {
  static int spmv_dot(const mgb_csr* a, const float* x, float* y, int i, int v, float* d) {
    return mgb_spmv_dot_csr_f32(a, x, y, i, v, d, nullptr);
  }
  static int cg(const mgb_csr* a, int v, const float* b, float* x, int64_t m, double t, int64_t* it, double* r) {
    return mgb_cg_csr_f32(a, v, b, x, m, t, it, r, nullptr);
  }
};
}  // namespace Impl

// y = A*x (init) or y += A*x, and returns x . y, in one pass over A.
template <class ExecSpace, class T>
T multiply_dot(const CsrMatrix<T>& A, const DenseVector<T>& x, DenseVector<T>& y, const bool init = true) {
  Impl::require_gb300<ExecSpace>();
  if ((int64_t)x.size() < A.ncols() || (int64_t)y.size() < A.nrows())
    throw InvalidInputException("multiply_dot: vector sizes do not match the matrix");
  DenseVector<T> d(1);
  mgb_csr desc = A.desc();
  Impl::check(Impl::SolverAbi<T>::spmv_dot(&desc, x.data(), y.data(), init, A.kernel_variant(), d.data()),
              "multiply_dot<GB300>");
  return d.to_host()[0];
}

struct CgResult {
  int64_t iterations;
  double relative_residual;  // sqrt(r.r / b.b) of the CG recurrence
};

// Conjugate gradients for an SPD CSR matrix; x holds the initial guess and
// receives the solution.  Throws RuntimeException if the matrix is not SPD.
template <class ExecSpace, class T>
CgResult cg(const CsrMatrix<T>& A, const DenseVector<T>& b, DenseVector<T>& x, int64_t max_iters, double rtol) {
  Impl::require_gb300<ExecSpace>();
  if (A.nrows() != A.ncols() || (int64_t)b.size() < A.nrows() || (int64_t)x.size() < A.nrows())
    throw InvalidInputException("cg: needs a square matrix and vectors of its size");
  CgResult r{0, 0.0};
  mgb_csr desc = A.desc();
  Impl::check(Impl::SolverAbi<T>::cg(&desc, A.kernel_variant(), b.data(), x.data(), max_iters, rtol, &r.iterations,
                                     &r.relative_residual),
              "cg<GB300>");
  return r;
}

// ------------------------------------------------------------- selector ---
// The learned format selector (an extension: the reference picks a format
// with the --morpheus-format flag, impl/Morpheus_Core.cpp:101-125).  Loads
// morpheus_gb300/selector_weights.bin (magic "MGBSEL01", u32 version, u32
// parameter count, u32 metadata length, mu[12], sigma[12], parameters,
// metadata; little-endian float32), computes the 12 features of the matrix
// on the GPU and runs the network's forward kernel; infeasible formats are
// never chosen.
class FormatSelector {
 public:
  explicit FormatSelector(const std::string& weights_path) {
    std::FILE* f = std::fopen(weights_path.c_str(), "rb");
    if (!f) throw IOException("cannot open " + weights_path);
    char magic[8];
    uint32_t head[3];
    const int n = mgb_mlp_num_params();
    std::vector<float> mu(12), sigma(12), params((size_t)n);
    const bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "MGBSEL01", 8) == 0 &&
                    std::fread(head, 4, 3, f) == 3 && head[0] == 1 && (int)head[1] == n &&
                    std::fread(mu.data(), 4, 12, f) == 12 && std::fread(sigma.data(), 4, 12, f) == 12 &&
                    std::fread(params.data(), 4, (size_t)n, f) == (size_t)n;
    std::fclose(f);
    if (!ok) throw IOException(weights_path + ": not a selector weights file of this library");
    for (auto& v : sigma) v = v < 1e-6f ? 1e-6f : v;
    params_.assign(params);
    mu_.assign(mu);
    sigma_.assign(sigma);
  }

  // The format the network picks for A (any container; its features are
  // computed in place, the same in every format).
  template <class T>
  formats_e select(const DiaMatrix<T>& A) const {
    std::vector<float> feat(12);
    std::vector<uint8_t> feas(6);
    const mgb_dia d = A.desc();
    Impl::check(Impl::features_of_typed<T>(&d, feat.data(), feas.data()), "FormatSelector::select");
    return pick(feat, feas);
  }
  template <class T>
  formats_e select(const HdcMatrix<T>& A) const {
    std::vector<float> feat(12);
    std::vector<uint8_t> feas(6);
    const mgb_hdc d = A.desc();
    Impl::check(Impl::features_of_typed<T>(&d, feat.data(), feas.data()), "FormatSelector::select");
    return pick(feat, feas);
  }
  template <class Matrix>
  formats_e select(const Matrix& A) const {  // CSR, COO, ELL, HYB
    std::vector<float> feat(12);
    std::vector<uint8_t> feas(6);
    const auto d = A.desc();
    Impl::check(Impl::features_of(&d, feat.data(), feas.data()), "FormatSelector::select");
    return pick(feat, feas);
  }

 private:
  formats_e pick(const std::vector<float>& feat, const std::vector<uint8_t>& feas) const {
    DeviceArray<float> X(feat), logp(6);
    DeviceArray<uint8_t> F(feas);
    Impl::check(mgb_mlp_forward_f32(params_.data(), mu_.data(), sigma_.data(), X.data(), F.data(), 1, logp.data(),
                                    nullptr),
                "FormatSelector::select");
    const std::vector<float> lp = logp.to_host();
    int best = CSR_FORMAT;
    for (int k = 0; k < 6; k++)
      if (feas[k] && (!feas[best] || lp[k] > lp[best])) best = k;
    return (formats_e)best;
  }
  DeviceArray<float> params_, mu_, sigma_;
};

// In-place switch of a DynamicMatrix to the format the selector picks.
template <class ExecSpace, class ValueType>
conversion_error_e convert(DynamicMatrix<ValueType>& A, const FormatSelector& selector) {
  const formats_e f = std::visit([&](const auto& m) { return selector.select(m); }, A.const_formats());
  return convert<ExecSpace>(A, f);
}

}  // namespace Morpheus

#endif  // MORPHEUS_GB300_HPP
