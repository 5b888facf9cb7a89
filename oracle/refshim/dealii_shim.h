// Minimal stand-in for the handful of deal.II types that pi-BEM's expansion
// sources (multipole_expansion.cc, local_expansion.cc, local_expansion_coeff.cc,
// ass_leg_function.cc, laplace_kernel.h) use: Point<3>, Tensor<1,3>,
// FullMatrix<double>, numbers::PI, Assert.  It lets those reference files be
// compiled unmodified so that their outputs can pin the oracle.  Test
// infrastructure only: nothing in the product links against it.
#ifndef PIBEM_ORACLE_DEALII_SHIM_H
#define PIBEM_ORACLE_DEALII_SHIM_H

#include <cmath>
#include <complex>
#include <cstring>
#include <iostream>
#include <map>
#include <set>
#include <string>
#include <vector>

namespace dealii
{
  namespace numbers
  {
    static const double PI = 3.14159265358979323846;
    static const unsigned int invalid_unsigned_int = static_cast<unsigned int>(-1);
  } // namespace numbers

  struct ExcInternalError
  {};

  template <int rank, int dim, typename Number = double>
  class Tensor;

  template <int dim, typename Number>
  class Tensor<1, dim, Number>
  {
  public:
    Number v[dim];
    Tensor()
    {
      for (int i = 0; i < dim; ++i)
        v[i] = 0;
    }
    Number &operator[](unsigned int i) { return v[i]; }
    const Number &operator[](unsigned int i) const { return v[i]; }
    Number norm() const { return std::sqrt(norm_square()); }
    Number norm_square() const
    {
      Number s = 0;
      for (int i = 0; i < dim; ++i)
        s += v[i] * v[i];
      return s;
    }
    Tensor &operator+=(const Tensor &o)
    {
      for (int i = 0; i < dim; ++i)
        v[i] += o.v[i];
      return *this;
    }
    Tensor &operator-=(const Tensor &o)
    {
      for (int i = 0; i < dim; ++i)
        v[i] -= o.v[i];
      return *this;
    }
    Tensor &operator*=(const Number s)
    {
      for (int i = 0; i < dim; ++i)
        v[i] *= s;
      return *this;
    }
    Tensor &operator/=(const Number s)
    {
      for (int i = 0; i < dim; ++i)
        v[i] /= s;
      return *this;
    }
  };

  template <int dim, typename Number = double>
  class Point : public Tensor<1, dim, Number>
  {
  public:
    Point() : Tensor<1, dim, Number>() {}
    Point(const Tensor<1, dim, Number> &t) : Tensor<1, dim, Number>(t) {}
    Point(Number x, Number y)
    {
      this->v[0] = x;
      this->v[1] = y;
    }
    Point(Number x, Number y, Number z)
    {
      this->v[0] = x;
      this->v[1] = y;
      if (dim > 2)
        this->v[2] = z;
    }
    Number operator()(unsigned int i) const { return this->v[i]; }
    Number &operator()(unsigned int i) { return this->v[i]; }
    Number square() const { return this->norm_square(); }
    Number distance(const Point &o) const
    {
      Number s = 0;
      for (int i = 0; i < dim; ++i)
        s += (this->v[i] - o.v[i]) * (this->v[i] - o.v[i]);
      return std::sqrt(s);
    }
    Point operator+(const Tensor<1, dim, Number> &o) const
    {
      Point r(*this);
      r += o;
      return r;
    }
    Tensor<1, dim, Number> operator-(const Point &o) const
    {
      Tensor<1, dim, Number> r(*this);
      r -= o;
      return r;
    }
    Point operator-() const
    {
      Point r(*this);
      r *= -1.0;
      return r;
    }
    Point operator/(const Number s) const
    {
      Point r(*this);
      r /= s;
      return r;
    }
    Point operator*(const Number s) const
    {
      Point r(*this);
      r *= s;
      return r;
    }
  };

  template <int dim, typename Number>
  inline Point<dim, Number> operator*(const Number s, const Point<dim, Number> &p)
  {
    return p * s;
  }

  template <int dim, typename Number>
  inline Tensor<1, dim, Number> operator/(const Tensor<1, dim, Number> &t, const Number s)
  {
    Tensor<1, dim, Number> r(t);
    r /= s;
    return r;
  }

  template <int dim, typename Number>
  inline Tensor<1, dim, Number> operator*(const Tensor<1, dim, Number> &t, const Number s)
  {
    Tensor<1, dim, Number> r(t);
    r *= s;
    return r;
  }

  template <int dim, typename Number>
  inline Number operator*(const Tensor<1, dim, Number> &a, const Tensor<1, dim, Number> &b)
  {
    Number s = 0;
    for (int i = 0; i < dim; ++i)
      s += a[i] * b[i];
    return s;
  }

  template <int dim, typename Number>
  inline std::ostream &operator<<(std::ostream &os, const Tensor<1, dim, Number> &t)
  {
    for (int i = 0; i < dim; ++i)
      os << t[i] << (i + 1 < dim ? " " : "");
    return os;
  }

  template <typename Number>
  class FullMatrix
  {
  public:
    FullMatrix() : m_(0), n_(0) {}
    FullMatrix(unsigned int m, unsigned int n) : m_(m), n_(n), a_(size_t(m) * n, Number(0)) {}
    Number &operator()(unsigned int i, unsigned int j) { return a_[size_t(i) * n_ + j]; }
    const Number &operator()(unsigned int i, unsigned int j) const { return a_[size_t(i) * n_ + j]; }
    unsigned int m() const { return m_; }
    unsigned int n() const { return n_; }

  private:
    unsigned int        m_, n_;
    std::vector<Number> a_;
  };
} // namespace dealii

#define Assert(cond, exc) \
  do                      \
    {                     \
    }                     \
  while (false)
#define AssertThrow(cond, exc) \
  do                           \
    {                          \
    }                          \
  while (false)

#endif
