// Bayesian optimisation of solver parameters (see bayes.h for the method and
// its sources).
#include "bayes.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <limits>

namespace qio
{
namespace
{
const double kLog2Pi = 1.8378770664093453;

// bounds of the hyperparameters, natural log, in normalised units (inputs in
// [0, 1], objectives standardised)
const double kSf2Lo = std::log(1e-2), kSf2Hi = std::log(1e2);
const double kEllLo = std::log(1e-2), kEllHi = std::log(1e1);
const double kSn2Lo = std::log(1e-6), kSn2Hi = std::log(1e-1);

double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

// Gaussian process on n points u (n x d) with standardised values y
struct Gp
{
  int d = 0, n = 0;
  std::vector<double> u, y;
  std::vector<char> pseudo;  // a believer's point: no observation noise
  double sf2 = 1, sn2 = 1e-3;
  std::vector<double> inv_l2;  // 1 / length scale^2
  std::vector<double> L;       // lower Cholesky factor of K, n x n
  std::vector<double> Kf;      // the signal part of K (lower triangle), n x n
  std::vector<double> alpha;   // K^-1 y

  void set_theta(const std::vector<double>& th)
  {
    sf2 = std::exp(th[0]);
    inv_l2.resize(d);
    for (int k = 0; k < d; k++) inv_l2[k] = std::exp(-2.0 * th[1 + k]);
    sn2 = std::exp(th[1 + d]);
  }
  double kern(const double* a, const double* b) const
  {
    double s = 0;
    for (int k = 0; k < d; k++)
    {
      const double t = a[k] - b[k];
      s += t * t * inv_l2[k];
    }
    return sf2 * std::exp(-0.5 * s);
  }
  // K = Kf + sn2 I, its factor and alpha; a failed factorisation retries with
  // a growing diagonal
  bool factor()
  {
    L.assign((size_t)n * n, 0.0);
    Kf.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j <= i; j++) Kf[(size_t)i * n + j] = kern(&u[(size_t)i * d], &u[(size_t)j * d]);
    for (int attempt = 0; attempt < 4; attempt++)
    {
      const double jitter = attempt == 0 ? 0.0 : sf2 * std::pow(10.0, -10 + 2 * attempt);
      bool ok = true;
      for (int i = 0; i < n && ok; i++)
        for (int j = 0; j <= i; j++)
        {
          double s = Kf[(size_t)i * n + j];
          if (i == j) s += ((i < (int)pseudo.size() && pseudo[i]) ? 1e-8 * sf2 : sn2) + jitter;
          for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
          if (i == j)
          {
            if (!(s > 0)) { ok = false; break; }
            L[(size_t)i * n + i] = std::sqrt(s);
          }
          else
            L[(size_t)i * n + j] = s / L[(size_t)j * n + j];
        }
      if (ok)
      {
        alpha = y;
        solve(alpha);
        return true;
      }
    }
    return false;
  }
  // v <- L^-1 v
  void fwd(std::vector<double>& v) const
  {
    for (int i = 0; i < n; i++)
    {
      double s = v[i];
      for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * v[k];
      v[i] = s / L[(size_t)i * n + i];
    }
  }
  // v <- L^-T v
  void bwd(std::vector<double>& v) const
  {
    for (int i = n - 1; i >= 0; i--)
    {
      double s = v[i];
      for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * v[k];
      v[i] = s / L[(size_t)i * n + i];
    }
  }
  void solve(std::vector<double>& v) const
  {
    fwd(v);
    bwd(v);
  }
  // posterior mean and variance of the latent function at x, with their
  // gradients in x when dmu is given
  void predict(const double* x, double& mu, double& var, double* dmu = nullptr, double* dvar = nullptr) const
  {
    std::vector<double> k(n);
    for (int i = 0; i < n; i++) k[i] = kern(x, &u[(size_t)i * d]);
    mu = 0;
    for (int i = 0; i < n; i++) mu += k[i] * alpha[i];
    std::vector<double> v = k;
    fwd(v);
    double q = 0;
    for (int i = 0; i < n; i++) q += v[i] * v[i];
    var = std::max(sf2 - q, 1e-12 * sf2);
    if (!dmu) return;
    bwd(v);  // K^-1 k
    for (int c = 0; c < d; c++)
    {
      double gm = 0, gv = 0;
      for (int i = 0; i < n; i++)
      {
        const double dk = -k[i] * (x[c] - u[(size_t)i * d + c]) * inv_l2[c];
        gm += alpha[i] * dk;
        gv += v[i] * dk;
      }
      dmu[c] = gm;
      dvar[c] = -2.0 * gv;
    }
  }
};

// log marginal likelihood of theta and its gradient
double lml(Gp& g, const std::vector<double>& th, std::vector<double>* grad)
{
  g.set_theta(th);
  if (!g.factor()) return -std::numeric_limits<double>::infinity();
  const int n = g.n, d = g.d;
  double v = 0;
  for (int i = 0; i < n; i++) v -= 0.5 * g.y[i] * g.alpha[i] + std::log(g.L[(size_t)i * n + i]);
  v -= 0.5 * n * kLog2Pi;
  if (!grad) return v;
  // W = alpha alpha^T - K^-1, with K^-1 = L^-T L^-1 from the triangular
  // inverse (lower triangles only: W and dK/dtheta are symmetric)
  std::vector<double> Li((size_t)n * n, 0.0), Kinv((size_t)n * n, 0.0);
  for (int j = 0; j < n; j++)
  {
    Li[(size_t)j * n + j] = 1.0 / g.L[(size_t)j * n + j];
    for (int i = j + 1; i < n; i++)
    {
      double s = 0;
      for (int k = j; k < i; k++) s -= g.L[(size_t)i * n + k] * Li[(size_t)k * n + j];
      Li[(size_t)i * n + j] = s / g.L[(size_t)i * n + i];
    }
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++)
    {
      double s = 0;
      for (int k = i; k < n; k++) s += Li[(size_t)k * n + i] * Li[(size_t)k * n + j];
      Kinv[(size_t)i * n + j] = s;
    }
  grad->assign(d + 2, 0.0);
  std::vector<double>& gr = *grad;
  for (int i = 0; i < n; i++)
    for (int j = 0; j <= i; j++)
    {
      const double m = i == j ? 0.5 : 1.0;  // off-diagonal pairs count twice
      const double w = m * (g.alpha[i] * g.alpha[j] - Kinv[(size_t)i * n + j]);
      const double* a = &g.u[(size_t)i * d];
      const double* b = &g.u[(size_t)j * d];
      const double kf = g.Kf[(size_t)i * n + j];
      gr[0] += w * kf;
      for (int c = 0; c < d; c++)
      {
        const double t = a[c] - b[c];
        gr[1 + c] += w * kf * t * t * g.inv_l2[c];
      }
      if (i == j) gr[1 + d] += w * g.sn2;
    }
  return v;
}

double norm_pdf(double z) { return 0.3989422804014327 * std::exp(-0.5 * z * z); }
double norm_cdf(double z) { return 0.5 * std::erfc(-z * 0.7071067811865476); }

// expected improvement below f (minimisation) and its gradient
double ei(const Gp& g, const double* x, double f, double* grad)
{
  const int d = g.d;
  std::vector<double> dmu(d), dvar(d);
  double mu, var;
  g.predict(x, mu, var, grad ? dmu.data() : nullptr, grad ? dvar.data() : nullptr);
  const double s = std::sqrt(var);
  const double z = (f - mu) / s;
  const double Phi = norm_cdf(z), phi = norm_pdf(z);
  if (grad)
    for (int c = 0; c < d; c++) grad[c] = -Phi * dmu[c] + phi * dvar[c] / (2.0 * s);
  return (f - mu) * Phi + s * phi;
}

// projected gradient ascent with an adaptive step on the box [lo, hi]^m;
// returns the best value reached, x updated in place
template <class F>
double ascend(F&& f, std::vector<double>& x, const std::vector<double>& lo, const std::vector<double>& hi,
              int steps, double eta)
{
  const size_t m = x.size();
  std::vector<double> g(m), xn(m), gn(m);
  double v = f(x, &g);
  if (!std::isfinite(v)) return v;
  for (int s = 0; s < steps && eta > 1e-6; s++)
  {
    double gmax = 0;
    for (double t : g) gmax = std::max(gmax, std::fabs(t));
    if (gmax == 0) break;
    const double scale = eta / std::max(1.0, gmax);
    for (size_t i = 0; i < m; i++) xn[i] = clampd(x[i] + scale * g[i], lo[i], hi[i]);
    const double vn = f(xn, &gn);
    if (std::isfinite(vn) && vn > v)
    {
      x = xn;
      g = gn;
      v = vn;
      eta = std::min(eta * 1.5, 4.0);
    }
    else
      eta *= 0.5;
  }
  return v;
}
}  // namespace

void BayesOpt::init(int dims, uint32_t seed)
{
  d_ = dims;
  xs_.clear();
  ys_.clear();
  xs_.reserve(reserved * dims);
  ys_.reserve(reserved);
  next_ = 0;
  best_ = 0;
  rng_ = 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed << 1);
  theta_.clear();
  winners_.clear();
  cur_ = num_to_sample;
  learning_ms = model_ms = 0;
}

// splitmix64 (Steele, Lea and Flood, OOPSLA 2014): the strategy's own draws
double BayesOpt::uniform()
{
  uint64_t z = (rng_ += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

void BayesOpt::add_sample(const std::vector<double>& x, double y)
{
  if (ys_.empty() || y < best_) best_ = y;
  if (ys_.size() < reserved)
  {
    ys_.push_back(y);
    xs_.insert(xs_.end(), x.begin(), x.begin() + d_);
  }
  else
  {
    // the reference scans as many slots as there are dimensions
    for (int i = 0; i < d_; i++)
    {
      const size_t r = (next_ + (size_t)i) % reserved;
      if (ys_[r] > y)
      {
        next_ = r;
        break;
      }
    }
    ys_[next_] = y;
    std::copy(x.begin(), x.begin() + d_, xs_.begin() + next_ * d_);
  }
  next_ = (next_ + 1) % reserved;
}

bool BayesOpt::recommend(std::vector<double>& out)
{
  out.assign(d_, 0.0);
  if (cur_ < num_to_sample && !winners_.empty())
  {
    std::copy(winners_.begin() + (size_t)cur_ * d_, winners_.begin() + (size_t)(cur_ + 1) * d_, out.begin());
    cur_++;
    return true;
  }
  const int n = (int)ys_.size();
  if (n < 2 || (int)ranges_.size() != d_) return false;
  const auto t0 = std::chrono::steady_clock::now();
  const int d = d_;
  Gp g;
  g.d = d;
  g.n = n;
  g.u.resize((size_t)n * d);
  std::vector<double> lo(d), span(d);
  for (int c = 0; c < d; c++)
  {
    lo[c] = ranges_[c].first;
    span[c] = ranges_[c].second - ranges_[c].first;
  }
  for (int i = 0; i < n; i++)
    for (int c = 0; c < d; c++)
      g.u[(size_t)i * d + c] = span[c] > 0 ? (xs_[(size_t)i * d + c] - lo[c]) / span[c] : 0.0;
  double mean = 0, sd = 0;
  for (double y : ys_) mean += y;
  mean /= n;
  for (double y : ys_) sd += (y - mean) * (y - mean);
  sd = std::sqrt(sd / n);
  if (!(sd > 1e-12 * std::max(1.0, std::fabs(mean)))) sd = 1.0;
  g.y.resize(n);
  for (int i = 0; i < n; i++) g.y[i] = (ys_[i] - mean) / sd;

  // hyperparameters: the previous fit and random starts in the bounds
  std::vector<double> tlo(d + 2), thi(d + 2);
  tlo[0] = kSf2Lo;
  thi[0] = kSf2Hi;
  for (int c = 0; c < d; c++)
  {
    tlo[1 + c] = kEllLo;
    thi[1 + c] = kEllHi;
  }
  tlo[1 + d] = kSn2Lo;
  thi[1 + d] = kSn2Hi;
  std::vector<double> th0(d + 2);
  if ((int)theta_.size() == d + 2)
    th0 = theta_;
  else
  {
    th0[0] = 0.0;
    for (int c = 0; c < d; c++) th0[1 + c] = std::log(0.3);
    th0[1 + d] = std::log(1e-3);
  }
  auto f_lml = [&](const std::vector<double>& th, std::vector<double>* gr) { return lml(g, th, gr); };
  double best_v = -std::numeric_limits<double>::infinity();
  std::vector<double> best_th;
  // later fits start from the previous one; the random starts matter less
  const int starts = n > 48 ? std::min(fit_starts, 3) : fit_starts;
  for (int s = 0; s < starts; s++)
  {
    std::vector<double> th(d + 2);
    if (s == 0)
      th = th0;
    else
      for (int i = 0; i < d + 2; i++) th[i] = tlo[i] + (thi[i] - tlo[i]) * uniform();
    for (int i = 0; i < d + 2; i++) th[i] = clampd(th[i], tlo[i], thi[i]);
    const double v = ascend(f_lml, th, tlo, thi, fit_steps, 1.0);
    if (v > best_v)
    {
      best_v = v;
      best_th = th;
    }
  }
  if (!std::isfinite(best_v)) return false;
  theta_ = best_th;
  g.set_theta(theta_);
  if (!g.factor()) return false;
  const auto t1 = std::chrono::steady_clock::now();
  model_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();

  // a batch by expected improvement, the process conditioned on each pick
  double fbest = g.y[0];
  for (double y : g.y) fbest = std::min(fbest, y);
  std::vector<double> ulo(d, 0.0), uhi(d, 1.0);
  winners_.assign((size_t)num_to_sample * d, 0.0);
  for (int q = 0; q < num_to_sample; q++)
  {
    auto f_ei = [&](const std::vector<double>& x, std::vector<double>* gr) {
      return ei(g, x.data(), fbest, gr ? gr->data() : nullptr);
    };
    std::vector<std::pair<double, std::vector<double>>> cand;
    cand.reserve(search_candidates + g.n);
    for (int s = 0; s < search_candidates; s++)
    {
      std::vector<double> x(d);
      for (int c = 0; c < d; c++) x[c] = uniform();
      cand.push_back({f_ei(x, nullptr), x});
    }
    for (int i = 0; i < g.n; i++)
    {
      std::vector<double> x(g.u.begin() + (size_t)i * d, g.u.begin() + (size_t)(i + 1) * d);
      for (int c = 0; c < d; c++) x[c] = clampd(x[c] + 0.01 * (uniform() - 0.5), 0.0, 1.0);
      cand.push_back({f_ei(x, nullptr), x});
    }
    const int top = std::min<int>(search_starts, (int)cand.size());
    std::partial_sort(cand.begin(), cand.begin() + top, cand.end(),
                      [](const std::pair<double, std::vector<double>>& a,
                         const std::pair<double, std::vector<double>>& b) { return a.first > b.first; });
    double bv = -1;
    std::vector<double> bx;
    for (int s = 0; s < top; s++)
    {
      std::vector<double> x = cand[s].second;
      const double v = ascend(f_ei, x, ulo, uhi, search_steps, 0.1);
      if (v > bv)
      {
        bv = v;
        bx = x;
      }
    }
    for (int c = 0; c < d; c++)
    {
      const double v = span[c] > 0 ? lo[c] + bx[c] * span[c] : lo[c];
      winners_[(size_t)q * d + c] = clampd(v, ranges_[c].first, std::max(ranges_[c].first, ranges_[c].second));
    }
    if (q + 1 < num_to_sample)
    {
      double mu, var;
      g.predict(bx.data(), mu, var);
      g.u.insert(g.u.end(), bx.begin(), bx.end());
      g.y.push_back(mu);
      fbest = std::min(fbest, mu);  // the believed value counts as observed
      g.pseudo.resize(g.n, 0);
      g.pseudo.push_back(1);
      g.n++;
      if (!g.factor())
      {
        // a pick on top of a sample: keep the batch found so far
        for (int r = q + 1; r < num_to_sample; r++)
          std::copy(winners_.begin() + (size_t)q * d, winners_.begin() + (size_t)(q + 1) * d,
                    winners_.begin() + (size_t)r * d);
        break;
      }
    }
  }
  learning_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  cur_ = 0;
  std::copy(winners_.begin(), winners_.begin() + d_, out.begin());
  cur_ = 1;
  return true;
}

bool bayes_recommend(int dims, const double* lo, const double* hi, int n, const double* xs, const double* ys,
                     uint32_t seed, int count, double* out)
{
  BayesOpt b;
  b.num_to_sample = std::max(1, count);
  b.init(dims, seed);
  std::vector<std::pair<double, double>> r(dims);
  for (int c = 0; c < dims; c++) r[c] = {lo[c], hi[c]};
  b.set_ranges(r);
  std::vector<double> x(dims);
  for (int i = 0; i < n; i++)
  {
    std::copy(xs + (size_t)i * dims, xs + (size_t)(i + 1) * dims, x.begin());
    b.add_sample(x, ys[i]);
  }
  for (int q = 0; q < count; q++)
  {
    if (!b.recommend(x)) return false;
    std::copy(x.begin(), x.end(), out + (size_t)q * dims);
  }
  return true;
}
}  // namespace qio
