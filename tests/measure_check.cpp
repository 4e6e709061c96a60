// The product's host measurement code (record_values, ChainAcc in lg_host.cpp) fed with the CPU
// oracle's per-sweep records, which the GPU parity tests show to be bit-identical to the GPU's.
// Built and run by tests/test_measurement.py, which compares the printed observables with exact
// diagonalization; so the whole measurement pipeline, including the normal estimators of
// DISABLE_IMPROVED_ESTIMATOR, is checked without a GPU.
//
//   measure_check dim L beta jxy jz h spin2 disable_improved therm sweeps seed
// prints one line per observable: "<name>\t<mean>\t<error>", then one line per value a
// worker plug-in pushes per sweep (record_scalars, what lg_fetch_values returns):
// "V\t<name>\t<plain mean over the measurement sweeps>".
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lg_host.h"

int lg_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  std::fprintf(stderr, "%s\n", buf);
  return code;
}

extern "C" {
struct orc_params {
  int dim;
  int L;
  double beta;
  double jxy, jz, h;
  double force_scatter;
  uint64_t seed;
  int random_spins;
  int deterministic_uf;
  int spin2;
};
void* orc_create(const orc_params* p);
void orc_destroy(void* h);
void orc_sweep(void* h, int n);
int orc_status(void* h);
int orc_num_records(void* h);
int orc_record_words();
void orc_get_records(void* h, uint64_t* out);
}

int main(int argc, char** argv) {
  if (argc != 12) {
    std::fprintf(stderr, "usage: measure_check dim L beta jxy jz h spin2 disable therm sweeps seed\n");
    return 2;
  }
  lg_params p;
  lg_params_default(&p);
  p.lattice = std::atoi(argv[1]);
  p.L = std::atoi(argv[2]);
  p.beta = std::atof(argv[3]);
  p.Jxy = std::atof(argv[4]);
  p.Jz = std::atof(argv[5]);
  p.h = std::atof(argv[6]);
  p.spin2 = std::atoi(argv[7]);
  p.disable_improved_estimator = std::atoi(argv[8]);
  const int therm = std::atoi(argv[9]), sweeps = std::atoi(argv[10]);
  ChainSpec s;
  if (s.init(p) != LG_OK) return 3;

  const orc_params q{p.lattice, p.L, p.beta, p.Jxy, p.Jz, p.h, 0.0,
                     (uint64_t)std::strtoull(argv[11], nullptr, 10), 1, 1, p.spin2};
  void* h = orc_create(&q);
  orc_sweep(h, therm + sweeps);
  if (orc_status(h)) return 4;
  const int n = orc_num_records(h), w = orc_record_words();
  if (w != lg::REC_WORDS || n != therm + sweeps) return 5;
  std::vector<uint64_t> rec((size_t)n * w);
  orc_get_records(h, rec.data());
  orc_destroy(h);

  ChainAcc acc;
  std::vector<double> vsum(LG_NUM_VALUES, 0.0), row(LG_NUM_VALUES);
  for (int i = therm; i < n; ++i) {
    acc.push(s, rec.data() + (size_t)i * w);
    record_scalars(s, rec.data() + (size_t)i * w, row.data());
    for (int k = 0; k < LG_NUM_VALUES; ++k) vsum[k] += row[k];
  }
  lg_obs o;
  acc.report(s, &o);
  for (int k = 0; k < LG_NUM_OBS; ++k)
    std::printf("%s\t%.17g\t%.17g\n", lg_obs_name(k), o.mean[k], o.error[k]);
  const uint64_t mask = value_mask(s);
  for (int k = 0; k < LG_NUM_VALUES; ++k)
    if (mask >> k & 1) std::printf("V\t%s\t%.17g\n", lg_value_name(k), vsum[k] / (double)(n - therm));
  return 0;
}
