// Finite-difference checks of the parameter-free strategy's analytic
// gradients (qiotoolkit_gb300/csrc/bayes.cc, included whole so that its
// internal functions are reachable): the log marginal likelihood in the
// hyperparameters and the expected improvement in the point.  Compiled and
// run by tests/test_bayes_cpu.py; prints the worst relative errors.
#include "../../qiotoolkit_gb300/csrc/bayes.cc"

#include <cstdio>
#include <random>

using namespace qio;

int main()
{
  std::mt19937 r(1);
  std::uniform_real_distribution<double> U(0, 1);
  const int d = 3;
  double worst_lml = 0, worst_ei = 0;
  for (int n : {7, 30})
  {
    Gp g;
    g.d = d;
    g.n = n;
    g.u.resize((size_t)n * d);
    for (auto& x : g.u) x = U(r);
    g.y.resize(n);
    for (int i = 0; i < n; i++) g.y[i] = std::sin(3 * g.u[i * d]) + g.u[i * d + 1] - 0.5;
    const std::vector<double> th = {0.3, std::log(0.4), std::log(0.7), std::log(0.2), std::log(1e-3)};
    std::vector<double> gr;
    lml(g, th, &gr);
    for (size_t k = 0; k < th.size(); k++)
    {
      std::vector<double> tp = th, tm = th;
      tp[k] += 1e-6;
      tm[k] -= 1e-6;
      const double fd = (lml(g, tp, nullptr) - lml(g, tm, nullptr)) / 2e-6;
      worst_lml = std::max(worst_lml, std::fabs(fd - gr[k]) / std::max(1.0, std::fabs(fd)));
    }
    g.set_theta(th);
    g.factor();
    double fbest = g.y[0];
    for (double y : g.y) fbest = std::min(fbest, y);
    for (int t = 0; t < 5; t++)
    {
      double x[d], gx[d];
      for (int c = 0; c < d; c++) x[c] = U(r);
      ei(g, x, fbest, gx);
      for (int c = 0; c < d; c++)
      {
        double xp[d], xm[d];
        for (int e = 0; e < d; e++) xp[e] = xm[e] = x[e];
        xp[c] += 1e-6;
        xm[c] -= 1e-6;
        const double fd = (ei(g, xp, fbest, nullptr) - ei(g, xm, fbest, nullptr)) / 2e-6;
        worst_ei = std::max(worst_ei, std::fabs(fd - gx[c]) / std::max(1e-3, std::fabs(fd)));
      }
    }
  }
  std::printf("lml %.3e ei %.3e\n", worst_lml, worst_ei);
  return 0;
}
