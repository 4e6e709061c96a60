// Drives the CPU oracle (oracle/looper_oracle.cpp, test infrastructure) through its C API for
// tests/test_host_sanitizers.py, which builds both with gcc's address, undefined-behaviour and
// float-cast-overflow sanitizers: every model family the parity tests use (chain, square and
// cubic; S = 1/2, 1, 3/2; antiferromagnetic, ferromagnetic, Ising, XY, field), with both
// union-find variants, and the standalone mode.
#include <cstdint>
#include <cstdio>
#include <vector>

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
void orc_standalone(unsigned L, double T, unsigned sweeps, unsigned therm, double* out,
                    double* speed);
}

int main() {
  struct Model { int dim, L; double beta, jxy, jz, h; int spin2; };
  const Model models[] = {
      {1, 8, 4.0, 1, 1, 0, 1},      {2, 6, 2.0, 1, 0.5, 0.3, 1}, {3, 4, 1.0, 1, 0.5, 0.3, 1},
      {1, 6, 2.0, -1, -0.5, 0.1, 1}, {1, 6, 2.0, 1, 0, 0, 1},     {1, 4, 2.0, 1, 1, 0, 2},
      {1, 4, 1.0, 1, 0.5, 0.2, 3},  {1, 5, 1.5, -1, -1, 0.1, 2}, {2, 4, 3.0, 0, 1, 0, 1},
      {1, 6, 0.3, 1, 1, 0.1, 3}};
  for (const Model& m : models) {
    for (int det = 0; det < 2; ++det) {
      const orc_params p{m.dim, m.L, m.beta, m.jxy, m.jz, m.h, 0.0, 17, 1, det, m.spin2};
      void* h = orc_create(&p);
      orc_sweep(h, 300);
      if (orc_status(h)) {
        std::printf("oracle status %d\n", orc_status(h));
        return 1;
      }
      std::vector<uint64_t> r((size_t)orc_num_records(h) * orc_record_words());
      orc_get_records(h, r.data());
      orc_destroy(h);
    }
  }
  double out[10], speed = 0;
  orc_standalone(8, 0.2, 4096, 512, out, &speed);
  std::printf("ok\n");
  return 0;
}
