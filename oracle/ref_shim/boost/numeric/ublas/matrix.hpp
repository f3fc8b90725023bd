// Minimal dense-matrix stand-in for the parts of boost::numeric::ublas that
// the reference TwoChNRG sources use (oracle build only): row-major matrix,
// prod/trans/herm, element-wise +,-, scalar scaling, diagonal vector ranges.
#ifndef ORACLE_SHIM_UBLAS_MATRIX_HPP
#define ORACLE_SHIM_UBLAS_MATRIX_HPP
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <ostream>
#include <vector>

namespace boost { namespace numeric { namespace ublas {

namespace shim_detail {
template <class T> inline T conj_of(const T& x) { return x; }
template <class T> inline std::complex<T> conj_of(const std::complex<T>& x) { return std::conj(x); }
}  // namespace shim_detail

template <class T>
class matrix {
 public:
  typedef T value_type;
  typedef std::size_t size_type;
  matrix() : r_(0), c_(0) {}
  matrix(size_type r, size_type c) : r_(r), c_(c), d_(r * c, T()) {}
  matrix(size_type r, size_type c, const T& v) : r_(r), c_(c), d_(r * c, v) {}
  template <class U>
  matrix(const matrix<U>& o) : r_(o.size1()), c_(o.size2()), d_(o.data().begin(), o.data().end()) {}
  size_type size1() const { return r_; }
  size_type size2() const { return c_; }
  T& operator()(size_type i, size_type j) { return d_[i * c_ + j]; }
  const T& operator()(size_type i, size_type j) const { return d_[i * c_ + j]; }
  void resize(size_type r, size_type c, bool preserve = true) {
    std::vector<T> nd(r * c, T());
    if (preserve)
      for (size_type i = 0; i < r && i < r_; ++i)
        for (size_type j = 0; j < c && j < c_; ++j) nd[i * c + j] = d_[i * c_ + j];
    d_.swap(nd); r_ = r; c_ = c;
  }
  void clear() { for (size_type k = 0; k < d_.size(); ++k) d_[k] = T(); }
  std::vector<T>& data() { return d_; }
  const std::vector<T>& data() const { return d_; }
  matrix& operator+=(const matrix& o) { for (size_type k = 0; k < d_.size(); ++k) d_[k] += o.d_[k]; return *this; }
  matrix& operator-=(const matrix& o) { for (size_type k = 0; k < d_.size(); ++k) d_[k] -= o.d_[k]; return *this; }
  template <class S> matrix& operator*=(const S& s) { for (size_type k = 0; k < d_.size(); ++k) d_[k] *= s; return *this; }
  template <class S> matrix& operator/=(const S& s) { for (size_type k = 0; k < d_.size(); ++k) d_[k] /= s; return *this; }
  template <class U = T>
  matrix<typename U::value_type> real() const {
    matrix<typename U::value_type> m(r_, c_);
    for (size_type k = 0; k < d_.size(); ++k) m.data()[k] = d_[k].real();
    return m;
  }

 private:
  size_type r_, c_;
  std::vector<T> d_;
};

template <class T> matrix<T> operator+(matrix<T> a, const matrix<T>& b) { a += b; return a; }
template <class T> matrix<T> operator-(matrix<T> a, const matrix<T>& b) { a -= b; return a; }
template <class T> matrix<T> operator-(const matrix<T>& a) { matrix<T> m(a); m *= T(-1); return m; }
template <class T, class S> matrix<T> operator*(matrix<T> a, const S& s) { a *= s; return a; }
template <class T, class S> matrix<T> operator*(const S& s, matrix<T> a) { a *= s; return a; }
template <class T, class S> matrix<T> operator/(matrix<T> a, const S& s) { a /= s; return a; }

template <class T> matrix<T> trans(const matrix<T>& a) {
  matrix<T> m(a.size2(), a.size1());
  for (std::size_t i = 0; i < a.size1(); ++i)
    for (std::size_t j = 0; j < a.size2(); ++j) m(j, i) = a(i, j);
  return m;
}
template <class T> matrix<T> herm(const matrix<T>& a) {
  matrix<T> m(a.size2(), a.size1());
  for (std::size_t i = 0; i < a.size1(); ++i)
    for (std::size_t j = 0; j < a.size2(); ++j) m(j, i) = shim_detail::conj_of(a(i, j));
  return m;
}
template <class T> matrix<T> conj(const matrix<T>& a) {
  matrix<T> m(a);
  for (std::size_t k = 0; k < m.data().size(); ++k) m.data()[k] = shim_detail::conj_of(m.data()[k]);
  return m;
}
template <class T> matrix<T> element_prod(const matrix<T>& a, const matrix<T>& b) {
  matrix<T> m(a);
  for (std::size_t k = 0; k < m.data().size(); ++k) m.data()[k] *= b.data()[k];
  return m;
}
template <class T, class U>
matrix<decltype(T() * U())> prod(const matrix<T>& a, const matrix<U>& b) {
  matrix<decltype(T() * U())> m(a.size1(), b.size2());
  for (std::size_t i = 0; i < a.size1(); ++i)
    for (std::size_t k = 0; k < a.size2(); ++k) {
      T aik = a(i, k);
      for (std::size_t j = 0; j < b.size2(); ++j) m(i, j) += aik * b(k, j);
    }
  return m;
}

template <class T> matrix<T>& noalias(matrix<T>& m) { return m; }

class range {
 public:
  range(std::size_t a, std::size_t b) : a_(a), b_(b) {}
  std::size_t start() const { return a_; }
  std::size_t size() const { return b_ > a_ ? b_ - a_ : 0; }
 private:
  std::size_t a_, b_;
};

// A vector running along (r.start()+k, c.start()+k): the diagonal when both
// ranges start at zero, which is how the reference forms traces.
template <class M>
class matrix_vector_range {
 public:
  typedef typename M::value_type value_type;
  matrix_vector_range(M& m, const range& r, const range& c) : m_(&m), r_(r), c_(c) {}
  std::size_t size() const { return r_.size() < c_.size() ? r_.size() : c_.size(); }
  value_type operator()(std::size_t k) const { return (*m_)(r_.start() + k, c_.start() + k); }
 private:
  M* m_;
  range r_, c_;
};

template <class M>
typename M::value_type sum(const matrix_vector_range<M>& v) {
  typename M::value_type s = typename M::value_type();
  for (std::size_t k = 0; k < v.size(); ++k) s += v(k);
  return s;
}

template <class T>
std::ostream& operator<<(std::ostream& os, const matrix<T>& m) {
  os << "[" << m.size1() << "," << m.size2() << "](";
  for (std::size_t i = 0; i < m.size1(); ++i) {
    os << "(";
    for (std::size_t j = 0; j < m.size2(); ++j) os << m(i, j) << (j + 1 < m.size2() ? "," : "");
    os << ")" << (i + 1 < m.size1() ? "," : "");
  }
  return os << ")";
}

}}}  // namespace boost::numeric::ublas
#endif
