// Driver of the worker plug-in of INTEGRATION.md (its source is included first, as
// gpu_path_integral.C, extracted from INTEGRATION.md by tests/test_plugin.py), with the stand-in
// ALPS types of tests/plugin_stub: the way parapack drives a worker.
//
//   plugin_main KEY=value ... [--save-at N]
// builds the parameters, runs the worker until progress() reaches 1, pushing into an
// ObservableSet, and prints one line per observable: "<name>\t<count>\t<mean>".  With --save-at N
// it also saves the worker after N sweeps, loads the dump into a second worker, runs both to the
// end and prints "resumed identical" if the second pushed exactly the values the first did.
#include <cstdio>
#include <cstring>
#include <string>

#include GPU_PLUGIN_SOURCE

int main(int argc, char** argv) {
  alps::Parameters p;
  long save_at = -1;
  for (int i = 1; i < argc; ++i) {
    if (std::strcmp(argv[i], "--save-at") == 0 && i + 1 < argc) { save_at = std::atol(argv[++i]); continue; }
    const char* eq = std::strchr(argv[i], '=');
    if (!eq) return 2;
    p.set(std::string(argv[i], eq - argv[i]), std::string(eq + 1));
  }
  try {
    gpu_pi_worker w(p);
    alps::ObservableSet obs;
    w.init_observables(p, obs);
    long mcs = 0;
    alps::ObservableSet obs2;
    std::vector<char> dump;
    while (w.progress() < 1.0) {
      if (mcs == save_at) {
        alps::ODump od;
        w.save(od);
        dump = od.bytes;
        obs2 = obs;
      }
      w.run(obs);
      ++mcs;
    }
    for (auto& kv : obs.data) {
      double s = 0;
      for (double x : kv.second) s += x;
      std::printf("%s\t%zu\t%.17g\n", kv.first.c_str(), kv.second.size(),
                  kv.second.empty() ? 0.0 : s / kv.second.size());
    }
    if (save_at >= 0) {
      gpu_pi_worker w2(p);
      alps::IDump id(dump);
      w2.load(id);
      while (w2.progress() < 1.0) w2.run(obs2);
      bool same = obs2.data == obs.data;
      std::printf("resumed %s\n", same ? "identical" : "different");
    }
  } catch (const std::exception& e) {
    std::printf("error\t%s\n", e.what());
    return 1;
  }
  return 0;
}
