// A C++ caller of the C ABI, written as the INTEGRATION.md bindings are:
// compiled against include/qio_gb300.h and linked with libqio_gb300.so by
// tests/test_integration.py.  Without arguments it runs the host-side paths
// (model construction, its properties, argument and params errors); with
// --gpu it also runs the model + solver binding and the whole-runner
// binding on the device and prints their costs.
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "qio_gb300.h"

static int failures = 0;
#define CHECK(cond, what)                                             \
  do                                                                  \
  {                                                                   \
    if (!(cond))                                                      \
    {                                                                 \
      std::printf("FAIL %s: %s\n", what, qio_last_error_message());  \
      failures++;                                                     \
    }                                                                 \
  } while (0)

int main(int argc, char** argv)
{
  const bool gpu = argc > 1 && std::strcmp(argv[1], "--gpu") == 0;
  // a ring of ten spins with ferromagnetic couplings, as the reference's
  // model tests build it
  std::vector<int64_t> off{0};
  std::vector<int32_t> ids;
  std::vector<double> coef;
  for (int i = 0; i < 10; i++)
  {
    ids.push_back(i);
    ids.push_back((i + 1) % 10);
    off.push_back((int64_t)ids.size());
    coef.push_back(-1.0);
  }
  qio_model* model = nullptr;
  CHECK(qio_model_create(QIO_ISING, 10, off.data(), ids.data(), coef.data(), &model) == QIO_OK,
        "model create");
  qio_model_info info;
  CHECK(qio_model_get_info(model, &info) == QIO_OK, "model info");
  CHECK(info.n_vars == 10 && info.n_terms == 10 && info.max_locality == 2, "model size");

  // error paths: the status codes and messages a binding surfaces
  qio_model* bad = nullptr;
  CHECK(qio_model_create(99, 10, off.data(), ids.data(), coef.data(), &bad) == QIO_INVALID_ARGUMENT,
        "unknown kind refused");
  CHECK(bad == nullptr, "no handle on error");
  CHECK(std::strlen(qio_last_error_message()) > 0, "error message set");
  std::vector<int32_t> dup{0, 0};
  std::vector<int64_t> doff{0, 2};
  std::vector<double> dc{1.0};
  CHECK(qio_model_create(QIO_ISING, 1, doff.data(), dup.data(), dc.data(), &bad) == QIO_INVALID_ARGUMENT,
        "duplicate ids refused");
  CHECK(std::string(qio_last_error_message()).find("Duplicated ids") != std::string::npos,
        "the reference's duplicate-id message");
  qio_solver* solver = nullptr;
  CHECK(qio_solver_create(model, "simulatedannealing.qiotoolkit", R"({"params": {"restarts": -1}})",
                          &solver) == QIO_INVALID_ARGUMENT,
        "bad params refused");
  CHECK(qio_solver_create(model, "no-such-solver", R"({"params": {}})", &solver) != QIO_OK,
        "unknown target refused");

  // the parameter-free search strategy on caller samples (host only): a
  // parabola in one dimension with its minimum at 2
  {
    const double lo[1] = {0.0}, hi[1] = {5.0};
    const double xs[5] = {0.0, 1.0, 3.0, 4.0, 5.0};
    double ys[5];
    for (int i = 0; i < 5; i++) ys[i] = (xs[i] - 2.0) * (xs[i] - 2.0);
    double pick[2] = {-1, -1};
    CHECK(qio_bayes_recommend(1, lo, hi, 5, xs, ys, 7, 2, pick) == QIO_OK, "strategy recommends");
    CHECK(pick[0] >= 0.0 && pick[0] <= 5.0 && pick[1] >= 0.0 && pick[1] <= 5.0, "picks in the box");
    CHECK(std::fabs(pick[0] - 2.0) < 1.0, "first pick near the minimum");
    CHECK(qio_bayes_recommend(1, lo, hi, 1, xs, ys, 7, 1, pick) == QIO_INVALID_ARGUMENT, "one sample refused");
  }

  if (gpu)
  {
    // binding 2: model + solver
    CHECK(qio_solver_create(model, "paralleltempering.qiotoolkit",
                            R"({"params": {"seed": 7, "sweeps": 200,
                                 "temperatures": {"type": "geometric", "initial": 0.05,
                                                  "final": 3.0, "count": 8}}})",
                            &solver) == QIO_OK,
          "solver create");
    CHECK(qio_solver_init(solver, nullptr) == QIO_OK, "solver init");
    CHECK(qio_solver_run(solver, nullptr) == QIO_OK, "solver run");
    char* result = nullptr;
    CHECK(qio_solver_result_json(solver, &result) == QIO_OK, "solver result");
    if (result) std::printf("solver result: %.120s\n", result);
    qio_free(result);
    qio_solver_destroy(solver);
    // binding 1: the whole runner
    const char* input = R"({"cost_function": {"type": "ising", "version": "1.0",
        "terms": [{"c": -1, "ids": [0, 1]}, {"c": -1, "ids": [1, 2]}, {"c": -1, "ids": [2, 0]}]}})";
    char* out = nullptr;
    CHECK(qio_run_json(input, R"({"params": {"seed": 1, "sweeps": 50, "restarts": 4}})",
                       "simulatedannealing.qiotoolkit", &out) == QIO_OK,
          "run json");
    if (out)
    {
      CHECK(std::strstr(out, "\"cost\":-3") != nullptr, "ground state of the triangle");
      std::printf("runner result: %.120s\n", out);
    }
    qio_free(out);
  }
  qio_model_destroy(model);
  std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
  return failures ? 1 : 0;
}
