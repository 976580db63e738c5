// Morpheus_GB300_MatrixMarket.hpp -- Matrix Market I/O for the GB300 front end.
//
//   Morpheus::IO::read_matrix_market_file(A, filename)    core/src/Morpheus_MatrixMarket.hpp:62-130
//   Morpheus::IO::write_matrix_market_file(A, filename)   core/src/Morpheus_MatrixMarket.hpp:132-190
//
// A is a CooMatrix<T>, a DynamicMatrix<T> whose active format is COO, or a
// DenseVector<T>.  The file is parsed on the host (base-1 indices checked
// and made base 0, symmetric matrices expanded with each off-diagonal entry
// mirrored right after itself, entries stably sorted by (row, column), as
// core/src/impl/Morpheus_MatrixMarket_Impl.hpp:101-249 does) and the arrays
// are then uploaded into the device container.  Malformed files throw
// IOException; complex data, hermitian and skew-symmetric matrices throw
// NotImplementedException; a DynamicMatrix not in COO throws
// RuntimeException.  Deliberate differences: symmetry "unsymmetric" reads as
// "general" (the reference replaces such a matrix by an unfilled one), and
// values are written with 17 significant digits so that a written file reads
// back bit-identically (the reference streams 6 digits).
#ifndef MORPHEUS_GB300_MATRIXMARKET_HPP
#define MORPHEUS_GB300_MATRIXMARKET_HPP

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <limits>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "Morpheus_GB300.hpp"

namespace Morpheus {
namespace IO {
namespace Impl {

struct Banner {
  std::string storage, type, symmetry;
};

inline std::vector<std::string> tokens_of(const std::string& line) {
  std::istringstream is(line);
  std::vector<std::string> t;
  for (std::string s; is >> s;) t.push_back(s);
  return t;
}

// core/src/impl/Morpheus_MatrixMarket_Impl.hpp:68-100
inline Banner read_banner(std::istream& in) {
  std::string line;
  std::getline(in, line);
  const std::vector<std::string> t = tokens_of(line);
  if (t.size() != 5 || t[0] != "%%MatrixMarket" || t[1] != "matrix")
    throw IOException("invalid MatrixMarket banner");
  Banner b{t[2], t[3], t[4]};
  if (b.storage != "array" && b.storage != "coordinate")
    throw IOException("invalid MatrixMarket storage format [" + b.storage + "]");
  if (b.type != "complex" && b.type != "real" && b.type != "integer" && b.type != "pattern")
    throw IOException("invalid MatrixMarket data type [" + b.type + "]");
  if (b.symmetry != "general" && b.symmetry != "symmetric" && b.symmetry != "unsymmetric" &&
      b.symmetry != "hermitian" && b.symmetry != "skew-symmetric")
    throw IOException("invalid MatrixMarket symmetry [" + b.symmetry + "]");
  return b;
}

// the size line after the comment lines
inline std::vector<std::string> size_line(std::istream& in) {
  std::string line;
  do {
    if (!std::getline(in, line)) throw IOException("unexpected EOF while reading MatrixMarket entries");
  } while (!line.empty() && line[0] == '%');
  return tokens_of(line);
}

inline int64_t to_int(const std::string& s) {
  try {
    size_t pos = 0;
    const long long v = std::stoll(s, &pos);
    if (pos != s.size()) throw IOException("invalid MatrixMarket integer [" + s + "]");
    return (int64_t)v;
  } catch (const std::logic_error&) {
    throw IOException("invalid MatrixMarket integer [" + s + "]");
  }
}

template <class T>
T read_value(std::istream& in) {
  T v{};
  if (!(in >> v)) throw IOException("unexpected EOF while reading MatrixMarket entries");
  return v;
}

template <class T>
void read_coordinate(std::istream& in, const Banner& b, int64_t& nrows, int64_t& ncols, std::vector<int32_t>& r,
                     std::vector<int32_t>& c, std::vector<T>& v) {
  const std::vector<std::string> t = size_line(in);
  if (t.size() != 3) throw IOException("invalid MatrixMarket coordinate format");
  nrows = to_int(t[0]);
  ncols = to_int(t[1]);
  const int64_t nnz = to_int(t[2]);
  if (b.type == "complex") throw NotImplementedException("Morpheus does not currently support complex matrices");
  std::vector<int64_t> ri((size_t)nnz), ci((size_t)nnz);
  std::vector<T> vals((size_t)nnz, T(1));
  for (int64_t n = 0; n < nnz; n++) {
    ri[n] = read_value<int64_t>(in);
    ci[n] = read_value<int64_t>(in);
    if (b.type != "pattern") vals[n] = read_value<T>(in);
  }
  if (nnz > 0) {
    const auto [rmin, rmax] = std::minmax_element(ri.begin(), ri.end());
    const auto [cmin, cmax] = std::minmax_element(ci.begin(), ci.end());
    if (*rmin < 1) throw IOException("found invalid row index (index < 1)");
    if (*cmin < 1) throw IOException("found invalid column index (index < 1)");
    if (*rmax > nrows) throw IOException("found invalid row index (index > num_rows)");
    if (*cmax > ncols) throw IOException("found invalid column index (index > num_columns)");
  }
  if (b.symmetry == "hermitian")
    throw NotImplementedException("MatrixMarket I/O does not currently support hermitian matrices");
  if (b.symmetry == "skew-symmetric")
    throw NotImplementedException("MatrixMarket I/O does not currently support skew-symmetric matrices");
  std::vector<int64_t> R, C;
  std::vector<T> V;
  R.reserve((size_t)nnz);
  C.reserve((size_t)nnz);
  V.reserve((size_t)nnz);
  for (int64_t n = 0; n < nnz; n++) {
    R.push_back(ri[n] - 1);
    C.push_back(ci[n] - 1);
    V.push_back(vals[n]);
    if (b.symmetry == "symmetric" && ri[n] != ci[n]) {
      R.push_back(ci[n] - 1);
      C.push_back(ri[n] - 1);
      V.push_back(vals[n]);
    }
  }
  std::vector<size_t> order(R.size());
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t z) { return R[a] != R[z] ? R[a] < R[z] : C[a] < C[z]; });
  r.resize(order.size());
  c.resize(order.size());
  v.resize(order.size());
  for (size_t k = 0; k < order.size(); k++) {
    r[k] = (int32_t)R[order[k]];
    c[k] = (int32_t)C[order[k]];
    v[k] = V[order[k]];
  }
}

// core/src/impl/Morpheus_MatrixMarket_Impl.hpp:251-316, for an n x 1 / 1 x n array
template <class T>
std::vector<T> read_array(std::istream& in, const Banner& b) {
  const std::vector<std::string> t = size_line(in);
  if (t.size() != 2) throw IOException("invalid MatrixMarket array format");
  const int64_t nr = to_int(t[0]), nc = to_int(t[1]);
  if (b.type == "pattern") throw NotImplementedException("pattern array MatrixMarket format is not supported");
  if (b.type == "complex") throw NotImplementedException("complex type is not supported");
  std::vector<T> out((size_t)(nr * nc));
  for (auto& e : out) e = (T)read_value<double>(in);
  if (b.symmetry != "general")
    throw NotImplementedException("only general array symmetric MatrixMarket format is supported");
  if (nr != 1 && nc != 1 && !out.empty())
    throw NotImplementedException("a dense array with more than one row and column needs a DenseMatrix");
  return out;
}

inline std::ifstream open_in(const std::string& filename) {
  std::ifstream in(filename);
  if (!in) throw IOException("failed to open " + filename);
  return in;
}

template <class T>
void write_coo(const CooMatrix<T>& A, const std::string& filename) {
  std::ofstream out(filename);
  if (!out) throw IOException("failed to open " + filename);
  const std::vector<int32_t> r = A.crow_indices().to_host(), c = A.ccolumn_indices().to_host();
  const std::vector<T> v = A.cvalues().to_host();
  out << "%%MatrixMarket matrix coordinate real general\n";
  out << A.nrows() << "\t" << A.ncols() << "\t" << A.nnnz() << "\n";
  out << std::setprecision(std::numeric_limits<T>::max_digits10);
  for (size_t k = 0; k < v.size(); k++) out << (r[k] + 1) << " " << (c[k] + 1) << " " << v[k] << "\n";
}

}  // namespace Impl

template <class T>
void read_matrix_market_file(CooMatrix<T>& A, const std::string& filename) {
  std::ifstream in = Impl::open_in(filename);
  const Impl::Banner b = Impl::read_banner(in);
  if (b.storage != "coordinate")
    throw IOException("only coordinate storage format is supported for reading a MatrixMarket file into "
                      "CooMatrix container");
  int64_t nr = 0, nc = 0;
  std::vector<int32_t> r, c;
  std::vector<T> v;
  Impl::read_coordinate(in, b, nr, nc, r, c, v);
  A = CooMatrix<T>(nr, nc, r, c, v);
}

template <class T>
void read_matrix_market_file(DynamicMatrix<T>& A, const std::string& filename) {
  if (A.active_index() != COO_FORMAT)
    throw RuntimeException("read_matrix_market_stream: The active state of a DynamicMatrix must be set to "
                           "Morpheus::COO_FORMAT before reading a MatrixMarket stream!");
  CooMatrix<T> coo;
  read_matrix_market_file(coo, filename);
  A = std::move(coo);
}

template <class T>
void read_matrix_market_file(DenseVector<T>& x, const std::string& filename) {
  std::ifstream in = Impl::open_in(filename);
  const Impl::Banner b = Impl::read_banner(in);
  if (b.storage != "array")
    throw IOException("only coordinate storage format is supported for reading a MatrixMarket file into "
                      "DenseVector container");
  x = DenseVector<T>(Impl::read_array<T>(in, b));
}

template <class T>
void write_matrix_market_file(const CooMatrix<T>& A, const std::string& filename) {
  Impl::write_coo(A, filename);
}

template <class T>
void write_matrix_market_file(const DynamicMatrix<T>& A, const std::string& filename) {
  if (A.active_index() != COO_FORMAT)
    throw RuntimeException("write_matrix_market_stream: The active state of a DynamicMatrix must be set to "
                           "Morpheus::COO_FORMAT before writing a MatrixMarket stream!");
  Impl::write_coo(std::get<CooMatrix<T>>(A.const_formats()), filename);
}

template <class T>
void write_matrix_market_file(const DenseVector<T>& x, const std::string& filename) {
  std::ofstream out(filename);
  if (!out) throw IOException("failed to open " + filename);
  const std::vector<T> v = x.to_host();
  out << "%%MatrixMarket matrix array real general\n" << v.size() << "\t1\n";
  out << std::setprecision(std::numeric_limits<T>::max_digits10);
  for (const T& e : v) out << e << "\n";
}

}  // namespace IO
}  // namespace Morpheus

#endif  // MORPHEUS_GB300_MATRIXMARKET_HPP
