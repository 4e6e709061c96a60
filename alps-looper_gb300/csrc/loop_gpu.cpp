// loop_gpu: looper's standalone loop program (standalone/loop.C with standalone/options.h) run on
// the GB300 engine through the C ABI of looper_gpu.h.
//
// The command line, defaults and output are those of the standalone program, so that a user of
// it can switch binaries: the S = 1/2 Heisenberg antiferromagnet (J = 1) on a periodic chain,
//   -l int     System Length             (default 8, must be even)
//   -t double  Temperature               (default 0.2, > 0)
//   -n int     MCS for Measurement       (default 65536, > 0; thermalization is n / 8)
//   -h         the option list
// all spins up at the start (loop.C:58-59) and seed 29833 (loop.C:50).  The parameters are
// echoed on stdout before the run, the five results after it as "name = mean +- error" and the
// speed in MCS/sec on stderr (loop.C:171-187).  An invalid parameter prints "invalid parameter"
// and the option list on stderr and exits with status 255, as the standalone program does.
//
// The engine's random streams are its own (Philox, not the standalone's Mersenne Twister), so
// results agree with the standalone program within their statistical errors, not digit for digit.
// The errors are binning errors (the largest level with at least 64 bins); the standalone
// program's are plain standard errors of the per-sweep values, which are smaller for correlated
// sweeps.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "looper_gpu.h"

namespace {

struct Options {
  unsigned length = 8;
  double temperature = 0.2;
  unsigned sweeps = 1u << 16;
  unsigned therm = (1u << 16) >> 3;
  bool valid = true;
  bool help = false;
};

void usage(std::ostream& os) {
  os << "[command line options]\n\n"
     << "  -l int     System Length\n"
     << "  -t double  Temperature\n"
     << "  -n int     MCS for Measurement\n"
     << "  -h         this help\n\n";
}

Options parse(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-h") { o.help = true; return o; }
    if ((a == "-l" || a == "-t" || a == "-n") && i + 1 < argc) {
      const char* v = argv[++i];
      if (a == "-l") o.length = (unsigned)std::atoi(v);
      else if (a == "-t") o.temperature = std::atof(v);
      else { o.sweeps = (unsigned)std::atoi(v); o.therm = o.sweeps >> 3; }
      continue;
    }
    o.valid = false;
    return o;
  }
  if (o.length % 2 == 1 || o.length < 2 || !(o.temperature > 0.0) || o.sweeps == 0) {
    std::cerr << "invalid parameter\n";
    o.valid = false;
  }
  return o;
}

int fail(const char* what, int rc) {
  char msg[512];
  lg_last_error(msg, sizeof(msg));
  std::cerr << what << " failed (" << rc << "): " << msg << "\n";
  return 1;
}

void line(const char* name, const lg_obs& o, int k) {
  std::cout << name << o.mean[k] << " +- " << o.error[k] << std::endl;
}

}  // namespace

int main(int argc, char** argv) {
  const Options o = parse(argc, argv);
  if (o.help) { usage(std::cout); return 255; }
  if (!o.valid) { usage(std::cerr); return 255; }
  std::cout << "System Length             = " << o.length << '\n'
            << "Temperature               = " << o.temperature << '\n'
            << "MCS for Thermalization    = " << o.therm << '\n'
            << "MCS for Measurement       = " << o.sweeps << '\n';

  lg_params p;
  lg_params_default(&p);
  p.lattice = LG_CHAIN;
  p.L = (int)o.length;
  p.T = o.temperature;
  p.beta = 0.0;
  p.J = 1.0;
  p.sweeps = o.sweeps;
  p.thermalization = o.therm;
  p.seed = 29833;
  p.init_spins = 0;
  lg_chain* c = nullptr;
  int rc = lg_create(&p, &c);
  if (rc != LG_OK) return fail("lg_create", rc);

  const auto start = std::chrono::steady_clock::now();
  rc = lg_run(c, (int64_t)o.therm + o.sweeps);
  lg_obs obs;
  if (rc == LG_OK) rc = lg_observables(c, &obs);
  const auto end = std::chrono::steady_clock::now();
  if (rc != LG_OK) { lg_destroy(c); return fail("lg_run", rc); }
  const double elapsed = std::chrono::duration<double>(end - start).count();
  std::cerr << "Speed = " << ((double)o.therm + o.sweeps) / elapsed << " MCS/sec\n";
  line("Number of Clusters        = ", obs, LG_OBS_NUM_CLUSTERS);
  line("Energy Density            = ", obs, LG_OBS_ENERGY_DENSITY);
  line("Uniform Susceptibility    = ", obs, LG_OBS_SUSCEPTIBILITY);
  line("Staggered Magnetization^2 = ", obs, LG_OBS_STAG_MAGNETIZATION2);
  line("Staggered Susceptibility  = ", obs, LG_OBS_STAG_SUSCEPTIBILITY);
  lg_destroy(c);
  return 0;
}
