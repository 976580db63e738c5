// test_frontend.cpp -- the C++17 front end (include/Morpheus_GB300.hpp) on the
// GPU, checked against the CPU oracle (oracle/liboracle.so, test
// infrastructure only).  The cases follow the reference's own tests:
//
//   multiply   core/tests/Test_Multiply.hpp:161-186,202-257 (banded matrices,
//              diagonals {0, +-5k}, N in {10, 100, 1000}, every format,
//              init and accumulate)
//   convert    core/tests/Serial/Test_Convert.hpp and
//              core/tests/Serial/Test_Convert_Dynamic.hpp:195-213
//              (structures bit-exact with the Serial convert, in-place
//              DynamicMatrix round trips, error codes)
//   dot        core/tests/Test_Dot.hpp:74-87   (sum (i+1)(n-i))
//   reduce     core/tests/Test_Reduce.hpp:74-81 (sum (i+1.5))
//   waxpby     core/tests/Test_WAXPBY.hpp
//   I/O        core/tests/Test_MatrixMarket.hpp (files written by this program
//              into the directory given as argv[1])
//
// Build: g++ -std=c++17 -Iinclude -I<cuda>/include tests/cpp/test_frontend.cpp
//        -Lmorpheus_gb300 -lmorpheus_gb300 -Loracle/_build -loracle -lcudart
// Exit status 0 when every check passes; one line per failed check.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "Morpheus_GB300.hpp"
#include "Morpheus_GB300_MatrixMarket.hpp"

extern "C" {
void* orc_new(int fmt, int dtype);
void orc_free(void* p);
int orc_resize(void* p, const int64_t* s);
int orc_shape(void* p, int64_t* s);
int64_t orc_array(void* p, const char* name, void** out);
int orc_convert(void* src, void* dst);
int orc_convert_inplace(void* p, int fmt);
int orc_sort_by_row_and_column(void* p);
int orc_multiply(void* p, const void* x, void* y, int init, int threads);
void orc_waxpby_f64(int64_t n, double a, const double* x, double b, const double* y, double* w);
}

namespace {

int g_checks = 0, g_failed = 0;

void expect(bool ok, const std::string& what) {
  ++g_checks;
  if (!ok) {
    ++g_failed;
    std::printf("FAIL: %s\n", what.c_str());
  }
}

template <class T> constexpr int dtype_code() { return std::is_same_v<T, double> ? 0 : 1; }
template <class T> const char* tname() { return std::is_same_v<T, double> ? "double" : "float"; }

// Host CSR of the reference's banded test matrix: diagonals 0 and +-k*freq,
// values U[-2, 2] (never 0) from a seeded generator of this file.
template <class T>
struct HostCsr {
  int64_t n = 0;
  std::vector<int32_t> ro, ci;
  std::vector<T> v;
};

template <class T>
HostCsr<T> banded(int64_t n, int64_t freq, unsigned seed) {
  HostCsr<T> h;
  h.n = n;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-2.0, 2.0);
  h.ro.push_back(0);
  for (int64_t i = 0; i < n; i++) {
    for (int64_t j = 0; j < n; j++) {
      const int64_t d = j - i;
      if (d % freq == 0) {
        double val = U(rng);
        if (val == 0.0) val = 1.0;
        h.ci.push_back((int32_t)j);
        h.v.push_back((T)val);
      }
    }
    h.ro.push_back((int32_t)h.ci.size());
  }
  return h;
}

template <class T>
std::vector<T> host_vector(int64_t n, unsigned seed) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::vector<T> x((size_t)n);
  for (auto& e : x) e = (T)U(rng);
  return x;
}

// ------------------------------------------------------------- oracle side
struct Oracle {
  void* h = nullptr;
  Oracle(int fmt, int dtype) : h(orc_new(fmt, dtype)) {}
  ~Oracle() { if (h) orc_free(h); }
  Oracle(const Oracle&) = delete;
  Oracle& operator=(const Oracle&) = delete;
  template <class E>
  std::vector<E> array(const char* name) const {
    void* p = nullptr;
    const int64_t n = orc_array(h, name, &p);
    if (n < 0) return {};
    const E* q = static_cast<const E*>(p);
    return std::vector<E>(q, q + n);
  }
  template <class E>
  void set(const char* name, const std::vector<E>& src) {
    void* p = nullptr;
    const int64_t n = orc_array(h, name, &p);
    if (n == (int64_t)src.size() && n > 0) std::memcpy(p, src.data(), sizeof(E) * (size_t)n);
  }
  std::vector<int64_t> shape() const {
    std::vector<int64_t> s(10);
    orc_shape(h, s.data());
    return s;
  }
};

template <class T>
void oracle_from_csr(Oracle& o, const HostCsr<T>& A) {
  int64_t s[10] = {1, A.n, A.n, (int64_t)A.v.size(), 0, 0, 0, 0, 0, 0};
  orc_resize(o.h, s);
  o.set("row_offsets", A.ro);
  o.set("column_indices", A.ci);
  o.set("values", A.v);
}

template <class T>
double rel_err(const std::vector<T>& y, const std::vector<T>& ref) {
  double num = 0, den = 0;
  for (size_t i = 0; i < y.size(); i++) {
    const double d = (double)y[i] - (double)ref[i];
    num += d * d;
    den += (double)ref[i] * (double)ref[i];
  }
  return den > 0 ? std::sqrt(num / den) : std::sqrt(num);
}

template <class T> double tol() { return std::is_same_v<T, double> ? 1e-12 : 1e-5; }

}  // namespace

namespace {

using Morpheus::GB300;

// bit-exact comparison of a device container with the oracle's container
template <class E>
bool same(const std::vector<E>& a, const std::vector<E>& b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), sizeof(E) * a.size()) == 0);
}

template <class T>
bool same_structure(const Morpheus::CooMatrix<T>& m, const Oracle& o, const std::string& p = "") {
  return same(m.crow_indices().to_host(), o.array<int32_t>((p + "row_indices").c_str())) &&
         same(m.ccolumn_indices().to_host(), o.array<int32_t>((p + "column_indices").c_str())) &&
         same(m.cvalues().to_host(), o.array<T>((p + "values").c_str()));
}
template <class T>
bool same_structure(const Morpheus::CsrMatrix<T>& m, const Oracle& o, const std::string& p = "") {
  return same(m.crow_offsets().to_host(), o.array<int32_t>((p + "row_offsets").c_str())) &&
         same(m.ccolumn_indices().to_host(), o.array<int32_t>((p + "column_indices").c_str())) &&
         same(m.cvalues().to_host(), o.array<T>((p + "values").c_str()));
}
template <class T>
bool same_structure(const Morpheus::DiaMatrix<T>& m, const Oracle& o, const std::string& p = "") {
  return same(m.cdiagonal_offsets().to_host(), o.array<int32_t>((p + "diagonal_offsets").c_str())) &&
         same(m.cvalues().to_host(), o.array<T>((p + "values").c_str()));
}
template <class T>
bool same_structure(const Morpheus::EllMatrix<T>& m, const Oracle& o, const std::string& p = "") {
  return same(m.ccolumn_indices().to_host(), o.array<int32_t>((p + "column_indices").c_str())) &&
         same(m.cvalues().to_host(), o.array<T>((p + "values").c_str()));
}
template <class T>
bool same_structure(const Morpheus::HybMatrix<T>& m, const Oracle& o) {
  return same_structure(m.cell(), o, "ell.") && same_structure(m.ccoo(), o, "coo.");
}
template <class T>
bool same_structure(const Morpheus::HdcMatrix<T>& m, const Oracle& o) {
  return same_structure(m.cdia(), o, "dia.") && same_structure(m.ccsr(), o, "csr.");
}
template <class T>
bool same_structure(const Morpheus::DynamicMatrix<T>& m, const Oracle& o) {
  return std::visit([&](const auto& a) { return same_structure(a, o); }, m.const_formats());
}

const char* kFormat[] = {"COO", "CSR", "DIA", "ELL", "HYB", "HDC"};

// Test_Multiply + Test_Convert_Dynamic: CSR -> every format in place on the
// GPU, structure against the Serial convert, multiply against the Serial
// multiply, then back to CSR.
template <class T>
void test_banded(int64_t n) {
  const HostCsr<T> h = banded<T>(n, 5, (unsigned)n);
  const std::string tag = std::string(tname<T>()) + " banded N=" + std::to_string(n);
  const Morpheus::CsrMatrix<T> A(n, n, h.ro, h.ci, h.v);
  const std::vector<T> xh = host_vector<T>(n, 1), y0 = host_vector<T>(n, 2);
  const Morpheus::DenseVector<T> x(xh);
  for (int f = 0; f < (int)Morpheus::NFORMATS; f++) {
    const std::string ft = tag + " -> " + kFormat[f];
    Oracle o(1, dtype_code<T>());
    oracle_from_csr(o, h);
    const int oc = orc_convert_inplace(o.h, f);

    Morpheus::DynamicMatrix<T> dyn(A);
    const Morpheus::conversion_error_e ec = Morpheus::convert<GB300>(dyn, f);
    expect((int)ec == oc, ft + ": conversion_error_e " + std::to_string((int)ec) + " vs " + std::to_string(oc));
    if (oc != Morpheus::CONV_SUCCESS) {
      expect(dyn.active_index() == Morpheus::CSR_FORMAT, ft + ": source kept after a failed conversion");
      continue;
    }
    expect(dyn.active_index() == f, ft + ": active format");
    expect(same_structure(dyn, o), ft + ": structure bit-exact with the Serial convert");

    for (int init = 1; init >= 0; init--) {
      std::vector<T> ref = y0;
      orc_multiply(o.h, xh.data(), ref.data(), init, 0);
      Morpheus::DenseVector<T> y(y0);
      if (init) Morpheus::multiply<GB300>(dyn, x, y);
      else Morpheus::multiply<GB300>(dyn, x, y, false);
      const double e = rel_err(y.to_host(), ref);
      expect(e <= tol<T>(), ft + (init ? " multiply" : " multiply (accumulate)") + ": rel err " + std::to_string(e));
    }

    // back to CSR through the generic convert(src, dst)
    Morpheus::CsrMatrix<T> back;
    Morpheus::convert<GB300>(dyn, back);
    Oracle ob(1, dtype_code<T>());
    orc_convert(o.h, ob.h);
    expect(same_structure(back, ob), ft + " -> CSR: structure bit-exact with the Serial convert");
  }
}

// Irregular square CSR: row lengths 0..60 from a seeded generator (about a
// fifth of the rows empty), distinct sorted columns, values U[-2, 2].
template <class T>
HostCsr<T> irregular(int64_t n, unsigned seed) {
  HostCsr<T> h;
  h.n = n;
  std::mt19937_64 rng(seed);
  std::uniform_int_distribution<int> L(0, 60);
  std::uniform_int_distribution<int64_t> Cdist(0, n - 1);
  std::uniform_real_distribution<double> U(-2.0, 2.0);
  h.ro.push_back(0);
  for (int64_t i = 0; i < n; i++) {
    int len = L(rng);
    len = len < 12 ? 0 : len;
    std::vector<int32_t> cols;
    for (int k = 0; k < len; k++) cols.push_back((int32_t)Cdist(rng));
    std::sort(cols.begin(), cols.end());
    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
    for (int32_t c : cols) {
      h.ci.push_back(c);
      h.v.push_back((T)U(rng));
    }
    h.ro.push_back((int32_t)h.ci.size());
  }
  return h;
}

// The chunk plan cached by CsrMatrix: the planned multiply gives y bit for
// bit equal to the unplanned lane-segment kernel, and writing new row
// offsets through row_offsets() drops the plan (the next multiply matches
// the Serial multiply of the new structure).
template <class T>
void test_chunk_plan() {
  const int64_t n = 60000;
  const std::string tag = std::string(tname<T>()) + " chunk plan";
  const HostCsr<T> h = irregular<T>(n, 77);
  Morpheus::CsrMatrix<T> A(n, n, h.ro, h.ci, h.v);
  expect(A.kernel_variant() == MGB_CSR_SEGMENTS, tag + ": lane-segment kernel chosen");
  const std::vector<T> xh = host_vector<T>(n, 5);
  const Morpheus::DenseVector<T> x(xh);
  Morpheus::DenseVector<T> y1(std::vector<T>((size_t)n, T(0))), y2(std::vector<T>((size_t)n, T(0)));
  Morpheus::multiply<GB300>(A, x, y1);
  const mgb_csr d = A.desc();
  int st;
  if constexpr (std::is_same_v<T, double>)
    st = mgb_spmv_csr_variant_f64(&d, x.data(), y2.data(), 1, MGB_CSR_SEGMENTS, nullptr);
  else
    st = mgb_spmv_csr_variant_f32(&d, x.data(), y2.data(), 1, MGB_CSR_SEGMENTS, nullptr);
  expect(st == MGB_SUCCESS, tag + ": unplanned call");
  expect(same(y1.to_host(), y2.to_host()), tag + ": planned y bit-identical to the unplanned kernel");
  int64_t entries = 0;
  expect(A.chunk_plan(&entries) != nullptr && entries >= 2, tag + ": plan cached");

  // same nnz, rows reversed: new row offsets written through the accessor
  HostCsr<T> r;
  r.n = n;
  r.ro.push_back(0);
  for (int64_t i = n - 1; i >= 0; i--) {
    for (int32_t k = h.ro[i]; k < h.ro[i + 1]; k++) {
      r.ci.push_back(h.ci[k]);
      r.v.push_back(h.v[k]);
    }
    r.ro.push_back((int32_t)r.ci.size());
  }
  A.row_offsets().assign(r.ro);
  A.column_indices().assign(r.ci);
  A.values().assign(r.v);
  Morpheus::multiply<GB300>(A, x, y1);
  Oracle o(1, dtype_code<T>());
  oracle_from_csr(o, r);
  std::vector<T> ref((size_t)n, T(0));
  orc_multiply(o.h, xh.data(), ref.data(), 1, 0);
  const double e = rel_err(y1.to_host(), ref);
  expect(e <= tol<T>(), tag + ": new row offsets after a cached plan, rel err " + std::to_string(e));
}

// in-place convert refused by the fill tolerance leaves the data in place
void test_convert_errors() {
  const int64_t n = 20000;  // ~n diagonals: N * ndiags > 1e8 and fill > 10, so DIA is refused
  HostCsr<double> h;
  h.n = n;
  std::mt19937_64 rng(7);
  h.ro.push_back(0);
  for (int64_t i = 0; i < n; i++) {  // diagonal + one random entry per row: ~n diagonals
    const int32_t j = (int32_t)(rng() % n);
    if (j < i) { h.ci.push_back(j); h.v.push_back(1.0); }
    h.ci.push_back((int32_t)i); h.v.push_back(2.0);
    if (j > i) { h.ci.push_back(j); h.v.push_back(1.0); }
    h.ro.push_back((int32_t)h.ci.size());
  }
  Morpheus::DynamicMatrix<double> dyn(Morpheus::CsrMatrix<double>(n, n, h.ro, h.ci, h.v));
  Oracle o(1, 0);
  oracle_from_csr(o, h);
  const int oc = orc_convert_inplace(o.h, Morpheus::DIA_FORMAT);
  const auto ec = Morpheus::convert<GB300>(dyn, Morpheus::DIA_FORMAT);
  expect(oc == Morpheus::PROXY_TO_DYNAMIC, "oracle refuses DIA for a scattered matrix");
  expect(ec == Morpheus::PROXY_TO_DYNAMIC, "convert<GB300>(dyn, DIA) returns PROXY_TO_DYNAMIC");
  expect(dyn.active_index() == Morpheus::CSR_FORMAT && dyn.nnnz() == (int64_t)h.v.size(),
         "matrix unchanged after PROXY_TO_DYNAMIC");
  expect(Morpheus::convert<GB300>(dyn, Morpheus::CSR_FORMAT) == Morpheus::CONV_SUCCESS, "same-format convert");

  bool threw = false;
  try {
    Morpheus::DiaMatrix<double> d;
    Morpheus::convert<GB300>(Morpheus::CsrMatrix<double>(n, n, h.ro, h.ci, h.v), d);
  } catch (const Morpheus::FormatConversionException&) {
    threw = true;
  }
  expect(threw, "convert<GB300>(csr, dia) throws FormatConversionException");

  threw = false;
  try {
    Morpheus::DenseVector<double> x(10), y(10);
    Morpheus::multiply<GB300>(dyn, x, y);
  } catch (const Morpheus::InvalidInputException&) {
    threw = true;
  }
  expect(threw, "multiply with short vectors throws InvalidInputException");
}

// DynamicMatrix::activate: empty container of the new format; the active
// format or an index past the last one changes nothing
void test_activate() {
  const HostCsr<double> h = banded<double>(50, 5, 3);
  Morpheus::DynamicMatrix<double> dyn(Morpheus::CsrMatrix<double>(50, 50, h.ro, h.ci, h.v));
  dyn.activate(Morpheus::CSR_FORMAT);
  expect(dyn.nnnz() == (int64_t)h.v.size(), "activate(active format) keeps the data");
  dyn.activate(17);
  expect(dyn.active_index() == Morpheus::CSR_FORMAT && dyn.nnnz() == (int64_t)h.v.size(),
         "activate(index past the last format) is a no-op");
  dyn.activate(Morpheus::ELL_FORMAT);
  expect(dyn.active_index() == Morpheus::ELL_FORMAT && dyn.nrows() == 0 && dyn.nnnz() == 0,
         "activate switches to an empty container");
}

// COO sort on the device against the Serial sort
void test_sort() {
  const int64_t n = 300, nnz = 5000;
  std::mt19937_64 rng(11);
  std::vector<int32_t> r(nnz), c(nnz);
  std::vector<double> v(nnz);
  for (int64_t k = 0; k < nnz; k++) {
    r[k] = (int32_t)(rng() % n);
    c[k] = (int32_t)(rng() % n);
    v[k] = (double)(k + 1);
  }
  Morpheus::CooMatrix<double> A(n, n, r, c, v);
  expect(!Morpheus::is_sorted<GB300>(A), "random COO is not sorted");
  Morpheus::sort_by_row_and_column<GB300>(A);
  expect(Morpheus::is_sorted<GB300>(A), "sorted after sort_by_row_and_column");
  Oracle o(0, 0);
  int64_t s[10] = {0, n, n, nnz, 0, 0, 0, 0, 0, 0};
  orc_resize(o.h, s);
  o.set("row_indices", r);
  o.set("column_indices", c);
  o.set("values", v);
  orc_sort_by_row_and_column(o.h);
  expect(same_structure(A, o), "device sort bit-exact with the Serial sort (stable on duplicates)");
}

template <class T>
void test_vector_ops() {
  const std::string tag = tname<T>();
  for (int64_t n : {1, 1000, 100000}) {
    std::vector<T> a((size_t)n), b((size_t)n), c((size_t)n);
    for (int64_t i = 0; i < n; i++) {
      a[i] = (T)(i + 1);
      b[i] = (T)(n - i);
      c[i] = (T)(i + 1.5);
    }
    const Morpheus::DenseVector<T> x(a), y(b), z(c);
    // sum_{i<n} (i+1)(n-i) = n(n+1)(n+2)/6
    const double dot_ref = (double)n * (n + 1) * (n + 2) / 6.0;
    const double d = (double)Morpheus::dot<GB300>((size_t)n, x, y);
    expect(std::fabs(d - dot_ref) <= (std::is_same_v<T, double> ? 0.0 : 1e-6 * dot_ref),
           tag + " dot known answer n=" + std::to_string(n));
    // sum_{i<n} (i+1.5) = n(n+2)/2
    const double red_ref = (double)n * (n + 2) / 2.0;
    const double s = (double)Morpheus::reduce<GB300>(z, (size_t)n);
    expect(std::fabs(s - red_ref) <= (std::is_same_v<T, double> ? 0.0 : 1e-6 * red_ref),
           tag + " reduce known answer n=" + std::to_string(n));
  }
  const int64_t n = 12345;
  const std::vector<T> a = host_vector<T>(n, 5), b = host_vector<T>(n, 6);
  Morpheus::DenseVector<T> x(a), y(b), w(n);
  Morpheus::waxpby<GB300>((size_t)n, (T)0.75, x, (T)-1.25, y, w);
  const std::vector<T> wh = w.to_host();
  bool ok = true;
  for (int64_t i = 0; i < n; i++) {
    const T ref = (T)0.75 * a[i] + (T)-1.25 * b[i];
    if (std::fabs((double)wh[i] - (double)ref) > 4 * std::numeric_limits<T>::epsilon() * (std::fabs((double)ref) + 1))
      ok = false;
  }
  expect(ok, tag + " waxpby");
}

template <class Exc>
bool throws_on(const std::string& path, const std::string& text) {
  {
    std::ofstream f(path);
    f << text;
  }
  try {
    Morpheus::CooMatrix<double> A;
    Morpheus::IO::read_matrix_market_file(A, path);
  } catch (const Exc&) {
    return true;
  } catch (...) {
    return false;
  }
  return false;
}

void test_matrix_market(const std::string& dir) {
  const std::string f = dir + "/general.mtx";
  {
    std::ofstream o(f);
    o << "%%MatrixMarket matrix coordinate real general\n% comment\n3 4 5\n3 4 -1.5\n1 1 1.25\n2 3 7\n"
         "1 4 2.5e-3\n2 1 -0.5\n";
  }
  Morpheus::CooMatrix<double> A;
  Morpheus::IO::read_matrix_market_file(A, f);
  expect(A.nrows() == 3 && A.ncols() == 4 && A.nnnz() == 5, "mm: sizes");
  expect(A.crow_indices().to_host() == std::vector<int32_t>({0, 0, 1, 1, 2}) &&
             A.ccolumn_indices().to_host() == std::vector<int32_t>({0, 3, 0, 2, 3}) &&
             A.cvalues().to_host() == std::vector<double>({1.25, 2.5e-3, -0.5, 7.0, -1.5}),
         "mm: general real file sorted, base 0");

  const std::string s = dir + "/sym.mtx";
  {
    std::ofstream o(s);
    o << "%%MatrixMarket matrix coordinate pattern symmetric\n3 3 2\n2 1\n3 3\n";
  }
  Morpheus::DynamicMatrix<double> dyn(Morpheus::CooMatrix<double>{});
  Morpheus::IO::read_matrix_market_file(dyn, s);
  const auto& B = std::get<Morpheus::CooMatrix<double>>(dyn.const_formats());
  expect(B.crow_indices().to_host() == std::vector<int32_t>({0, 1, 2}) &&
             B.ccolumn_indices().to_host() == std::vector<int32_t>({1, 0, 2}),
         "mm: symmetric pattern expanded");

  const std::string bad = dir + "/bad.mtx";
  expect(throws_on<Morpheus::IOException>(bad, "%%MatrixMarket matrix coordinate real general symmetric\n1 1 0\n"),
         "mm: banner with an extra word");
  expect(throws_on<Morpheus::IOException>(bad, "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1\n"),
         "mm: zero row index");
  expect(throws_on<Morpheus::IOException>(bad, "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 3 1\n"),
         "mm: column index past ncols");
  expect(throws_on<Morpheus::IOException>(bad, "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n"),
         "mm: unexpected EOF");
  expect(throws_on<Morpheus::NotImplementedException>(bad,
                                                      "%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n"),
         "mm: complex");
  expect(throws_on<Morpheus::NotImplementedException>(bad,
                                                      "%%MatrixMarket matrix coordinate real hermitian\n1 1 1\n1 1 1\n"),
         "mm: hermitian");

  bool threw = false;
  try {
    Morpheus::DynamicMatrix<double> d(Morpheus::CsrMatrix<double>{});
    Morpheus::IO::read_matrix_market_file(d, f);
  } catch (const Morpheus::RuntimeException&) {
    threw = true;
  }
  expect(threw, "mm: DynamicMatrix must be in COO");

  // write -> read is bit-exact
  const HostCsr<double> h = banded<double>(300, 7, 9);
  Morpheus::CooMatrix<double> C;
  Morpheus::convert<GB300>(Morpheus::CsrMatrix<double>(300, 300, h.ro, h.ci, h.v), C);
  Morpheus::IO::write_matrix_market_file(C, dir + "/w.mtx");
  Morpheus::CooMatrix<double> D;
  Morpheus::IO::read_matrix_market_file(D, dir + "/w.mtx");
  expect(D.crow_indices().to_host() == C.crow_indices().to_host() &&
             D.ccolumn_indices().to_host() == C.ccolumn_indices().to_host() &&
             D.cvalues().to_host() == C.cvalues().to_host(),
         "mm: write -> read round trip bit-exact");
  const Morpheus::DenseVector<float> x(host_vector<float>(33, 3));
  Morpheus::IO::write_matrix_market_file(x, dir + "/x.mtx");
  Morpheus::DenseVector<float> z;
  Morpheus::IO::read_matrix_market_file(z, dir + "/x.mtx");
  expect(z.to_host() == x.to_host(), "mm: vector round trip bit-exact");
}

// fused SpMV + dot equals multiply + dot; CG solves an SPD system
void test_solver() {
  const int64_t n = 4000;
  HostCsr<double> h;
  h.n = n;
  h.ro.push_back(0);
  for (int64_t i = 0; i < n; i++) {  // symmetric, diagonally dominant: SPD
    for (int64_t d : {-9, -1, 0, 1, 9}) {
      const int64_t j = i + d;
      if (j < 0 || j >= n) continue;
      h.ci.push_back((int32_t)j);
      h.v.push_back(d == 0 ? 4.5 : -1.0);
    }
    h.ro.push_back((int32_t)h.ci.size());
  }
  const Morpheus::CsrMatrix<double> A(n, n, h.ro, h.ci, h.v);
  const std::vector<double> bh = host_vector<double>(n, 21);
  const Morpheus::DenseVector<double> b(bh);
  Morpheus::DenseVector<double> y(n), y2(n);
  const double d = Morpheus::multiply_dot<GB300>(A, b, y);
  Morpheus::multiply<GB300>(A, b, y2);
  expect(y.to_host() == y2.to_host(), "multiply_dot: y bit-identical to multiply");
  const double d2 = Morpheus::dot<GB300>((size_t)n, b, y2);
  expect(std::fabs(d - d2) <= 1e-12 * std::fabs(d2), "multiply_dot: dot matches dot<GB300>");

  Morpheus::DenseVector<double> x(n, 0.0);
  const Morpheus::CgResult r = Morpheus::cg<GB300>(A, b, x, 1000, 1e-11);
  expect(r.iterations > 0 && r.iterations < 1000 && r.relative_residual <= 1e-11, "cg converges");
  Oracle o(1, 0);
  oracle_from_csr(o, h);
  std::vector<double> ax(n, 0.0);
  const std::vector<double> xh = x.to_host();
  orc_multiply(o.h, xh.data(), ax.data(), 1, 0);
  double num = 0, den = 0;
  for (int64_t i = 0; i < n; i++) {
    num += (bh[i] - ax[i]) * (bh[i] - ax[i]);
    den += bh[i] * bh[i];
  }
  expect(std::sqrt(num / den) <= 1e-9, "cg: true residual against the oracle multiply");
}

// the learned selector from C++: a stencil goes to a diagonal format, a
// power-law-like matrix stays row-based, and the switch keeps the product
void test_selector(const std::string& weights) {
  const Morpheus::FormatSelector sel(weights);
  const int64_t n = 40;  // 40^3 7-point stencil
  HostCsr<double> h;
  h.n = n * n * n;
  h.ro.push_back(0);
  for (int64_t i = 0; i < n; i++)
    for (int64_t j = 0; j < n; j++)
      for (int64_t k = 0; k < n; k++) {
        const int64_t r = (i * n + j) * n + k;
        const int64_t nb[7][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
        for (const auto& d : nb) {
          const int64_t a = i + d[0], b = j + d[1], c = k + d[2];
          if (a < 0 || a >= n || b < 0 || b >= n || c < 0 || c >= n) continue;
          h.ci.push_back((int32_t)((a * n + b) * n + c));
          h.v.push_back(d[0] == 0 && d[1] == 0 && d[2] == 0 ? 6.0 : -1.0);
        }
        (void)r;
        h.ro.push_back((int32_t)h.ci.size());
      }
  const Morpheus::CsrMatrix<double> A(h.n, h.n, h.ro, h.ci, h.v);
  const Morpheus::formats_e f = sel.select(A);
  expect(f >= Morpheus::COO_FORMAT && f < Morpheus::NFORMATS, "selector returns a format");
  Morpheus::DynamicMatrix<double> dyn(A);
  expect(Morpheus::convert<GB300>(dyn, sel) == Morpheus::CONV_SUCCESS && dyn.active_index() == f,
         "convert(dyn, selector) switches to the selected format");
  const std::vector<double> xh = host_vector<double>(h.n, 31);
  Morpheus::DenseVector<double> x(xh), y(h.n), y2(h.n);
  Morpheus::multiply<GB300>(dyn, x, y);
  Morpheus::multiply<GB300>(A, x, y2);
  expect(rel_err(y.to_host(), y2.to_host()) <= 1e-12, "multiply after the selector's switch");
  bool threw = false;
  try {
    Morpheus::FormatSelector bad("/nonexistent/weights.bin");
  } catch (const Morpheus::IOException&) {
    threw = true;
  }
  expect(threw, "missing weights file throws IOException");
}

}  // namespace

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  const std::string weights = argc > 2 ? argv[2] : "";
  try {
    for (int64_t n : {10, 100, 1000}) {
      test_banded<double>(n);
      test_banded<float>(n);
    }
    test_chunk_plan<double>();
    test_chunk_plan<float>();
    test_convert_errors();
    test_activate();
    test_sort();
    test_vector_ops<double>();
    test_vector_ops<float>();
    test_matrix_market(dir);
    test_solver();
    if (!weights.empty()) test_selector(weights);
  } catch (const std::exception& e) {
    std::printf("FAIL: unexpected exception: %s\n", e.what());
    return 2;
  }
  std::printf("%d checks, %d failed\n", g_checks, g_failed);
  return g_failed == 0 ? 0 : 1;
}
