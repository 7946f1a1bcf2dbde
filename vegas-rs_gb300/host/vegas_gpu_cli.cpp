// vegas_gpu_cli -- the vegas command line (src/main.rs) on the GPU engine.
//
//   vegas_gpu_cli input                          print the default input
//   vegas_gpu_cli bench <ising|heisenberg> <L> [-s seed]
//   vegas_gpu_cli run <input.toml | -> [-s seed]
//
// `bench` is src/main.rs:24-59: sc lattice L^3 (full PBC), bare Exchange
// (J = 1), MetropolisIntegrator for both models, CoolDown::default() with
// max temperature 5.0 (Ising) / 2.5 (Heisenberg) and rate 0.05, StatSensor
// on stdout.  Errors print "Error: ..." and exit with status 1
// (src/main.rs:84-89).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>

#include "vegas/vegas.hpp"

using namespace vegas;

static uint64_t seed_or_random(bool has, uint64_t s) {
  if (has) return s;
  std::random_device rd;
  return ((uint64_t)rd() << 32) ^ rd();
}

template <typename S>
static void bench_model(int length, uint64_t seed, double max_t) {
  const Lattice lattice = Lattice::sc(1.0).expand_all(length);
  const Exchange H = Exchange::from_lattice(1.0, lattice);
  const CoolDown program = CoolDown().set_max_temperature(max_t).set_cool_rate(0.05);
  typename Machine<Exchange, GpuIntegrator, S>::Instruments instruments;
  instruments.push_back(std::make_unique<StatSensor<S>>(stdout));
  Machine<Exchange, GpuIntegrator, S> machine(Thermostat<S>(2.8, Field<S>::zero()), H, MetropolisIntegrator(seed),
                                             std::move(instruments), State<S>::up_with_size(lattice.sites_len()));
  check(vg_init_random(machine.context()), machine.context());
  program.run(machine);
}

int main(int argc, char** argv) {
  try {
    if (argc < 2) {
      std::fprintf(stderr, "usage: %s input | bench <ising|heisenberg> <L> [-s seed] | run <file|-> [-s seed]\n", argv[0]);
      return 2;
    }
    const std::string cmd = argv[1];
    bool has_seed = false;
    uint64_t seed = 0;
    std::vector<std::string> pos;
    for (int i = 2; i < argc; ++i) {
      if ((!std::strcmp(argv[i], "-s") || !std::strcmp(argv[i], "--seed")) && i + 1 < argc) {
        has_seed = true;
        seed = std::stoull(argv[++i]);
      } else {
        pos.push_back(argv[i]);
      }
    }
    if (cmd == "input") {
      std::fputs(Input::default_text().c_str(), stdout);
      return 0;
    }
    if (cmd == "bench" && pos.size() == 2) {
      const int L = std::stoi(pos[1]);
      if (pos[0] == "ising" || pos[0] == "Ising") bench_model<IsingSpin>(L, seed_or_random(has_seed, seed), 5.0);
      else if (pos[0] == "heisenberg" || pos[0] == "Heisenberg")
        bench_model<HeisenbergSpin>(L, seed_or_random(has_seed, seed), 2.5);
      else throw VegasError("unknown model " + pos[0]);
      return 0;
    }
    if (cmd == "run" && pos.size() == 1) {
      std::stringstream buf;
      if (pos[0] == "-") {
        buf << std::cin.rdbuf();
      } else {
        std::ifstream f(pos[0]);
        if (!f) throw IoError("std io error: cannot open " + pos[0]);
        buf << f.rdbuf();
      }
      Input::parse(buf.str()).run(seed_or_random(has_seed, seed));
      return 0;
    }
    std::fprintf(stderr, "usage: %s input | bench <ising|heisenberg> <L> [-s seed] | run <file|-> [-s seed]\n", argv[0]);
    return 2;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "Error: %s\n", e.what());
    return 1;
  }
}
