// Bayesian optimisation of solver parameters over a box: the search strategy
// of the population-annealing and substochastic parameter-free solvers (the
// role of strategy/bayesian.h:14-78 and strategy/bayesian.cc).
//
// A Gaussian process with a squared-exponential covariance models the
// objective (a run's lowest cost) over the parameter vectors sampled so far.
// Its hyperparameters (signal variance, one length scale per dimension,
// noise variance) maximise the log marginal likelihood (Rasmussen and
// Williams, Gaussian Processes for Machine Learning, 2006, eqs. 2.30 and
// 5.9) by projected gradient ascent from several starts.  The next points
// maximise expected improvement (Jones, Schonlau and Welch, J. Global
// Optimization 13, 1998); a batch of `num_to_sample` points is chosen one
// after another, the process conditioned on each chosen point at its
// predicted mean (the "kriging believer" of Ginsbourger, Le Riche and
// Carraro, Computational Intelligence in Expensive Optimization Problems,
// 2010).  The batch is handed out one point per call, as
// BayesianOpt::recommend_parameter_values does.  Host code: O(n^3) in the
// samples kept (at most `reserved` of them).
#pragma once

#include <cstdint>
#include <utility>
#include <vector>

namespace qio
{
class BayesOpt
{
 public:
  // training budget of the hyperparameter fit and of the point search
  int fit_starts = 6, fit_steps = 60;
  int search_candidates = 256, search_starts = 6, search_steps = 50;
  int num_to_sample = 4;
  size_t reserved = 128;

  void init(int dims, uint32_t seed);
  void set_ranges(const std::vector<std::pair<double, double>>& r) { ranges_ = r; }
  // the next point to run; false when the process could not be fitted
  // (the caller then falls back to its own update)
  bool recommend(std::vector<double>& out);
  // a finished run: its parameters and objective.  Past `reserved` samples a
  // new one replaces the oldest sample (from the last replacement on) whose
  // objective is worse (strategy/bayesian.cc:97-144)
  void add_sample(const std::vector<double>& x, double y);

  size_t n_samples() const { return ys_.size(); }
  double best() const { return best_; }
  const std::vector<double>& hyper() const { return theta_; }
  double learning_ms = 0, model_ms = 0;

 private:
  int d_ = 0;
  std::vector<std::pair<double, double>> ranges_;
  std::vector<double> xs_, ys_;  // samples, row-major n x d
  size_t next_ = 0;
  double best_ = 0;
  uint64_t rng_ = 0;
  std::vector<double> theta_;    // log sf2, log l[d], log sn2 (normalised units)
  std::vector<double> winners_;  // the last batch, num_to_sample x d
  int cur_ = 0;

  double uniform();
};

// one-call use of the strategy for callers outside the solvers: a fitted
// recommendation from samples (dims x n row-major), n >= 2
bool bayes_recommend(int dims, const double* lo, const double* hi, int n, const double* xs,
                     const double* ys, uint32_t seed, int count, double* out);
}  // namespace qio
