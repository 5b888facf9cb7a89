// C entry points over pi-BEM's own expansion classes (compiled unmodified from
// the reference sources): source/ass_leg_function.cc, source/multipole_expansion.cc,
// source/local_expansion.cc.  Used only to generate and check golden vectors for
// the oracle; never linked into the product.
//
// Coefficient arrays are the reference's complex triangular storage
// (index n(n+1)/2+m, include/multipole_expansion.h:102-105) flattened as
// interleaved (re, im) doubles: 2*(p+1)(p+2)/2 values.
#include "local_expansion.h"
#include "multipole_expansion.h"

namespace
{
  const AssLegFunction &alf()
  {
    static AssLegFunction a;
    return a;
  }
  unsigned ncoef(unsigned p) { return (p + 1) * (p + 2) / 2; }
  Point<3> pt(const double *x) { return Point<3>(x[0], x[1], x[2]); }

  template <class E>
  void load(E &e, unsigned p, const double *c)
  {
    for (unsigned i = 0; i < ncoef(p); ++i)
      e.GetCoeffs()[i] = std::complex<double>(c[2 * i], c[2 * i + 1]);
    e.is_zero = false;
  }
  template <class E>
  void store(const E &e, unsigned p, double *c)
  {
    for (unsigned i = 0; i < ncoef(p); ++i)
      {
        c[2 * i]     = e.GetCoeffs()[i].real();
        c[2 * i + 1] = e.GetCoeffs()[i].imag();
      }
  }
} // namespace

extern "C"
{
  double ref_legendre(unsigned n, unsigned m, double x) { return alf().GetAssLegFunSph(n, m, x); }
  double ref_legendre_deriv(unsigned n, unsigned m, double x)
  {
    return alf().GetAssLegFunSphDeriv(n, m, x);
  }

  // MultipoleExpansion::Add(strength, point) for each point (monopoles).
  void ref_p2m(unsigned p, const double *center, int npts, const double *pts, const double *q,
               double *out)
  {
    MultipoleExpansion e(p, pt(center), &alf());
    for (int i = 0; i < npts; ++i)
      e.Add(q[i], pt(pts + 3 * i));
    store(e, p, out);
  }

  // MultipoleExpansion::AddNormDer(strength, point, normal) (normal dipoles).
  void ref_p2m_dipole(unsigned p, const double *center, int npts, const double *pts,
                      const double *normals, const double *q, double *out)
  {
    MultipoleExpansion e(p, pt(center), &alf());
    for (int i = 0; i < npts; ++i)
      {
        Tensor<1, 3> n;
        n[0] = normals[3 * i];
        n[1] = normals[3 * i + 1];
        n[2] = normals[3 * i + 2];
        e.AddNormDer(q[i], pt(pts + 3 * i), n);
      }
    store(e, p, out);
  }

  // MultipoleExpansion::Add(child): M2M from child centre to parent centre.
  void ref_m2m(unsigned p, const double *c_child, const double *coef_child,
               const double *c_parent, double *out)
  {
    MultipoleExpansion child(p, pt(c_child), &alf());
    load(child, p, coef_child);
    MultipoleExpansion parent(p, pt(c_parent), &alf());
    parent.Add(child);
    store(parent, p, out);
  }

  // LocalExpansion::Add(multipole): M2L.
  void ref_m2l(unsigned p, const double *c_src, const double *coef_src, const double *c_tgt,
               double *out)
  {
    MultipoleExpansion m(p, pt(c_src), &alf());
    load(m, p, coef_src);
    LocalExpansion l(p, pt(c_tgt), &alf());
    l.Add(m);
    store(l, p, out);
  }

  // LocalExpansion::Add(parent local): L2L.
  void ref_l2l(unsigned p, const double *c_parent, const double *coef_parent,
               const double *c_child, double *out)
  {
    LocalExpansion par(p, pt(c_parent), &alf());
    load(par, p, coef_parent);
    LocalExpansion ch(p, pt(c_child), &alf());
    ch.Add(par);
    store(ch, p, out);
  }

  // MultipoleExpansion::Evaluate (M2P).
  double ref_m2p(unsigned p, const double *center, const double *coef, const double *x)
  {
    MultipoleExpansion m(p, pt(center), &alf());
    load(m, p, coef);
    return m.Evaluate(pt(x));
  }

  // LocalExpansion::Evaluate (L2P).
  double ref_l2p(unsigned p, const double *center, const double *coef, const double *x)
  {
    LocalExpansion l(p, pt(center), &alf());
    load(l, p, coef);
    return l.Evaluate(pt(x));
  }
}
