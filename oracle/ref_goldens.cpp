// Runs pi-BEM's own expansion classes (compiled unmodified from the reference
// sources) through the scenarios of the reference's golden-output tests and
// prints the same "DEAL::" log, so that the build can be checked line-for-line
// against the reference's committed .output files:
//   tests/multipole_expansion_creation_and_evaluation.cc
//   tests/multipole_expansion_translation.cc
//   tests/local_expansion_creation_and_evaluation.cc
//   tests/local_expansion_translation.cc
//   tests/multipole_expansion_creation_and_evaluation_neumann_kernel.cc
//   tests/multipole_expansion_copy.cc, tests/local_expansion_copy.cc
// Usage: ref_goldens <scenario>   (scenario = file stem of the test)
// Test infrastructure only.
#include <iomanip>
#include <sstream>

#include "local_expansion.h"
#include "multipole_expansion.h"

namespace
{
  // deallog stand-in: prefixes every line with "DEAL::", 6 significant digits
  // with trailing zeros kept, as deal.II's test log prints doubles.
  struct Log
  {
    std::ostringstream line;
    Log() { line << std::showpoint << std::setprecision(6); }
    template <typename T>
    Log &operator<<(const T &v)
    {
      line << v;
      return *this;
    }
    Log &operator<<(std::ostream &(*)(std::ostream &))
    {
      std::cout << "DEAL::" << line.str() << "\n";
      line.str("");
      return *this;
    }
  } deallog;

  std::ostream &operator<<(std::ostream &os, const std::complex<double> &c)
  {
    return os << "(" << c.real() << "," << c.imag() << ")";
  }

  struct Charges
  {
    std::vector<Point<3>> x;
    std::vector<double>   q;
    std::vector<Point<3>> n;
  };

  Charges five_charges()
  {
    Charges c;
    c.x = {Point<3>(2.8, 3.0, 3.0), Point<3>(3.0, 2.8, 3.0), Point<3>(3.0, 3.0, 2.8),
           Point<3>(3.2, 3.0, 3.0), Point<3>(3.0, 3.0, 3.2)};
    c.q = {0.1, 0.4, 1.0, 0.2, 0.7};
    return c;
  }

  double log_charges(const Charges &c)
  {
    Point<3> zero(0.0, 0.0, 0.0);
    double   exact = 0.0;
    for (unsigned int i = 0; i < c.x.size(); ++i)
      {
        exact += c.q[i] / c.x[i].distance(zero);
        deallog << "Charge " << i + 1 << " of intensity " << c.q[i] << " is located at point ("
                << c.x[i] << ")" << std::endl;
      }
    return exact;
  }

  void log_result(double exact, double approx)
  {
    deallog << "Approx potential at point Q(0,0,0): " << approx << std::endl;
    deallog << "The absolute multipole approximation error is: " << std::fabs(exact - approx)
            << std::endl;
    deallog << "The relative multipole approximation error is: "
            << std::fabs(exact - approx) / std::fabs(exact) << std::endl;
  }
} // namespace

int main(int argc, char **argv)
{
  const std::string which = argc > 1 ? argv[1] : "";
  std::cout << "\n"; // the reference's .output files open with an empty line
  AssLegFunction   *alf   = new AssLegFunction();
  const unsigned    p     = 6;
  Point<3>          zero(0.0, 0.0, 0.0);
  Point<3>          center(3.0, 3.0, 3.0);

  if (which == "multipole_expansion_creation_and_evaluation_neumann_kernel")
    {
      Charges c;
      c.x = {Point<3>(2.8, 3.0, 3.0), Point<3>(3.0, 2.8, 3.0), Point<3>(3.2, 3.0, 2.8),
             Point<3>(3.2, 3.0, 3.0), Point<3>(2.7, 3.0, 3.2)};
      c.q = {0.1, 0.4, 1.0, 0.2, 0.7};
      c.n.assign(5, Point<3>(1.0, 0.0, 0.0));
      double exact = 0.0;
      for (unsigned int i = 0; i < 5; ++i)
        {
          exact += -c.q[i] * (c.x[i] * c.n[i]) / std::pow(c.x[i].distance(zero), 3.0);
          deallog << "Charge " << i + 1 << " of intensity " << c.q[i] << " is located at point ("
                  << c.x[i] << ")  and has normal (" << c.n[i] << ")" << std::endl;
        }
      deallog << "Exact potential normal gradient at point Q(0,0,0): " << exact << std::endl;
      MultipoleExpansion mp(p, center, alf);
      for (unsigned int i = 0; i < 5; ++i)
        mp.AddNormDer(c.q[i], c.x[i], c.n[i]);
      log_result(exact, mp.Evaluate(zero));
      return 0;
    }

  Charges c     = five_charges();
  double  exact = log_charges(c);
  MultipoleExpansion mp(p, center, alf);
  if (which == "multipole_expansion_copy" || which == "local_expansion_copy")
    {
      for (unsigned int i = 0; i < 5; ++i)
        mp.Add(c.q[i], c.x[i]);
      std::complex<double> diff(0., 0.);
      if (which == "multipole_expansion_copy")
        {
          MultipoleExpansion copy(mp);
          for (unsigned int i = 0; i < (p + 1) * (p + 2) / 2; ++i)
            diff += mp.GetCoeffs()[i] - copy.GetCoeffs()[i];
          deallog << "Original and copied multipole  are created. " << std::endl;
          deallog << "" << std::endl;
          deallog << "Total difference between original and copied multipole expansion entries: "
                  << diff << std::endl;
        }
      else
        {
          LocalExpansion local(p, Point<3>(-2.0, -2.0, -2.0), alf);
          local.Add(mp);
          LocalExpansion copy(local);
          for (unsigned int i = 0; i < (p + 1) * (p + 2) / 2; ++i)
            diff += local.GetCoeffs()[i] - copy.GetCoeffs()[i];
          deallog << "Original and copied local expansions are created. " << std::endl;
          deallog << "" << std::endl;
          deallog << "Total difference between original and copied local expansion entries: "
                  << diff << std::endl;
        }
      return 0;
    }

  deallog << "Exact potential at point Q(0,0,0): " << exact << std::endl;
  for (unsigned int i = 0; i < 5; ++i)
    mp.Add(c.q[i], c.x[i]);
  double approx = 0.0;
  if (which == "multipole_expansion_creation_and_evaluation")
    approx = mp.Evaluate(zero);
  else if (which == "multipole_expansion_translation")
    {
      MultipoleExpansion parent(p, Point<3>(4.0, 4.0, 4.0), alf);
      parent.Add(mp);
      approx = parent.Evaluate(zero);
    }
  else if (which == "local_expansion_creation_and_evaluation")
    {
      LocalExpansion local(p, Point<3>(-2.0, -2.0, -2.0), alf);
      local.Add(mp);
      approx = local.Evaluate(zero);
    }
  else if (which == "local_expansion_translation")
    {
      LocalExpansion local(p, Point<3>(-2.0, -2.0, -2.0), alf);
      local.Add(mp);
      LocalExpansion local2(p, Point<3>(-1.0, -1.0, -1.0), alf);
      local2.Add(local);
      approx = local2.Evaluate(zero);
    }
  else
    {
      std::cerr << "unknown scenario " << which << "\n";
      return 2;
    }
  log_result(exact, approx);
  return 0;
}
