// host_selftest -- checks of the C++ host mirror.
//
//   host_selftest --cpu   logic that needs no GPU: schedules, accumulator,
//                         StatSensor format, TOML input, program errors,
//                         hamiltonian descriptors
//   host_selftest --gpu DIR   Machine + programs + instruments on the engine
//                             (instrument files under DIR)
//   host_selftest --parquet-demo DIR   writes DIR/demo.parquet (3 row groups
//                             of the observables schema) for a reader check
//
// Prints one line per check and exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vegas/vegas.hpp"

using namespace vegas;

static int g_checks = 0;
#define CHECK(cond)                                                            \
  do {                                                                         \
    ++g_checks;                                                                \
    if (!(cond)) {                                                             \
      std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);     \
      std::exit(1);                                                            \
    }                                                                          \
  } while (0)

template <typename F>
static bool throws_program_error(F f, ProgramError::Kind k) {
  try {
    f();
  } catch (const ProgramError& e) {
    return e.kind == k;
  }
  return false;
}

static std::string slurp(FILE* f) {
  std::string s;
  std::rewind(f);
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
  return s;
}

static int count_lines(const std::string& s) {
  int n = 0;
  for (char c : s) n += c == '\n';
  return n;
}

static void snappy_checks() {
  // round trips of the page compressor over its element kinds: literals of
  // every length class, short and long copies, overlapping runs, far offsets
  std::vector<std::vector<uint8_t>> cases;
  cases.push_back({});
  cases.push_back({42});
  std::vector<uint8_t> run(100000, 7);
  cases.push_back(run);
  std::vector<uint8_t> text;
  for (int i = 0; i < 5000; ++i) {
    const char* w = (i % 7 == 0) ? "magnetization " : (i % 3 == 0) ? "energy " : "step ";
    text.insert(text.end(), w, w + std::strlen(w));
  }
  cases.push_back(text);
  uint64_t x = 88172645463325252ull;
  std::vector<uint8_t> noise(300000);
  for (auto& b : noise) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    b = (uint8_t)x;
  }
  cases.push_back(noise);
  std::vector<uint8_t> far = noise;  // a repeat 100 KB back: four-byte offsets
  far.insert(far.end(), noise.begin(), noise.begin() + 70000);
  cases.push_back(far);
  std::vector<uint8_t> doubles;  // PLAIN float64 / uint64 columns as the observables write them
  for (int i = 0; i < 20000; ++i) {
    const double d = -1.0 * (i / 7);
    const uint64_t u = (uint64_t)(i / 3);
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&d);
    doubles.insert(doubles.end(), p, p + 8);
    const uint8_t* q = reinterpret_cast<const uint8_t*>(&u);
    doubles.insert(doubles.end(), q, q + 8);
  }
  cases.push_back(doubles);
  for (const auto& c : cases) {
    const std::vector<uint8_t> z = snappy::compress(c);
    CHECK(snappy::decompress(z.data(), z.size()) == c);
  }
  CHECK(snappy::compress(run).size() < run.size() / 20);
  CHECK(snappy::compress(doubles).size() < doubles.size() / 2);
}

static void cpu_checks() {
  snappy_checks();
  // CoolDown / HysteresisLoop schedules (src/program.rs:202-211, :302-332)
  CHECK(CoolDown(4.0, 0.1, 0.1).temperatures().size() == 39);
  CHECK(CoolDown(5.5, 3.5, 0.1).temperatures().size() == 21);
  CHECK(CoolDown(2.0, 0.2, 0.1).temperatures().size() == 18);
  CHECK(CoolDown().set_max_temperature(5.0).set_cool_rate(0.05).temperatures().size() == 100);
  CHECK(HysteresisLoop(1, 1, 1.0, 5.0, 0.1).fields().size() == 255);
  // program validation (src/program.rs:105-110, :190-201, :289-300)
  CHECK(throws_program_error([] { CoolDown(1.0, 2.0).validate(); }, ProgramError::Kind::TemperatureMaxLessThanMin));
  CHECK(throws_program_error([] { CoolDown(3.0, 0.05, 0.1, 10, 0).validate(); }, ProgramError::Kind::NoSteps));
  CHECK(throws_program_error([] { CoolDown(3.0, 0.0).validate(); }, ProgramError::Kind::ZeroTemperature));
  CHECK(throws_program_error([] { CoolDown(3.0, 0.1, 0.0).validate(); }, ProgramError::Kind::ZeroCoolRate));
  CHECK(throws_program_error([] { HysteresisLoop(1, 1, 1.0, 0.0).validate(); }, ProgramError::Kind::ZeroField));
  CHECK(throws_program_error([] { HysteresisLoop(1, 1, 1.0, 1.0, 0.0).validate(); },
                             ProgramError::Kind::ZeroFieldStep));
  // accumulator (src/accumulator.rs:42-63)
  Accumulator a;
  for (double x : {1.0, 2.0, 3.0, 4.0}) a.collect(x);
  CHECK(a.mean() == 2.5);
  CHECK(a.variance() == 7.5 - 6.25);
  CHECK(std::fabs(a.binder_cumulant() - (1.0 - 88.5 / (3.0 * 7.5 * 7.5))) < 1e-15);
  // thermostat clamp and field magnitude (src/thermostat.rs:29-39, src/state.rs:219-221)
  CHECK(Thermostat<IsingSpin>(0.0, Field<IsingSpin>::zero()).temperature() == kEpsilon);
  CHECK(Field<HeisenbergSpin>(HeisenbergSpin::up(), -2.0).magnitude() == 2.0);
  // state magnetization (src/state.rs:344-350)
  CHECK(State<IsingSpin>::up_with_size(10).magnetization().magnitude() == 10.0);
  CHECK(State<HeisenbergSpin>::down_with_size(4).magnetization().orientation.sz() == -1.0);
  // hamiltonian! nesting and descriptors
  const Lattice l = Lattice::sc(1.0).expand(4, 4, 1).drop_z();
  const auto h1 = describe(Exchange::from_lattice(2.0, l));
  CHECK(h1.compound == 0 && h1.has_exchange && h1.exchange == 2.0);
  const auto h3 = describe(hamiltonian(Exchange::from_lattice(1.0, l), UniaxialAnisotropy<HeisenbergSpin>(HeisenbergSpin::up(), 0.1),
                                       Zeeman<HeisenbergSpin>()));
  CHECK(h3.compound == 1 && h3.has_anisotropy && h3.anisotropy == 0.1 && h3.zeeman_sign == 1.0);
  CHECK(l.sites_len() == 16 && l.desc().pbc_z == 0);
  // StatSensor line format: 7 columns with 16 decimals (src/instrument.rs:113-123)
  FILE* f = std::tmpfile();
  StatSensor<IsingSpin> ss(f);
  ss.on_measure_start(Thermostat<IsingSpin>(2.0, Field<IsingSpin>::zero()), 4);
  for (double e : {-8.0, -6.0}) ss.after_step(StepView<IsingSpin>{e, 4.0, 4, nullptr});
  ss.on_measure_end();
  const std::string line = slurp(f);
  std::fclose(f);
  CHECK(line == "2.0000000000000000 0.0000000000000000 -7.0000000000000000 0.0625000000000000 4.0000000000000000 "
                "0.0000000000000000 0.6666666666666667\n");
  // TOML input (the shape of docs/metropolis.toml)
  const Input in = Input::parse(
      "model = \"Ising\"\nalgorithm = \"Metropolis\"\n# comment\n[sample.unitcell]\nname = \"bcc\"\n"
      "[sample.size]\nx = 10\ny = 8\nz = 6\n[sample.pbc]\nx = true\ny = false\nz = true\n"
      "[[stages]]\nprogram = \"Relax\"\nsteps = 100\ntemperature = 6.0\n"
      "[[stages]]\nprogram = \"CoolDown\"\nmax_temperature = 6.0\nmin_temperature = 1.0\ncool_rate = 0.05\n"
      "relax = 10\nsteps = 20\n[output]\nobservables = \"./o.csv\"\n[output.state]\npath = \"./s.csv\"\nfrequency = 7\n");
  CHECK(in.unitcell == "bcc" && in.size[0] == 10 && in.size[2] == 6 && !in.pbc[1]);
  CHECK(in.stages.size() == 2 && in.observables == "./o.csv" && in.state_frequency == 7);
  CHECK(in.lattice().sites_len() == 2u * 10 * 8 * 6 && in.lattice().desc().pbc_y == 0);
  const Input def = Input::parse(Input::default_text());
  CHECK(def.stages.size() == 2 && def.model == "Ising");
  bool bad = false;
  try {
    Input::parse("model = \"Potts\"\nalgorithm = \"Metropolis\"\n");
  } catch (const TomlError&) {
    bad = true;
  }
  CHECK(bad);
  bool wolff = false;
  try {
    Input w = def;
    w.algorithm = "Wolff";
    w.model = "Heisenberg";  // (Heisenberg, Wolff) is not implemented (src/input.rs:365)
    w.run(1, stdout);
  } catch (const NotImplementedError&) {
    wolff = true;
  }
  CHECK(wolff);
}

static void gpu_checks(const std::string& dir) {
  int32_t ndev = 0;
  vg_device_count(&ndev);
  CHECK(ndev > 0);
  // CoolDown on a 2D Ising lattice with StatSensor + ObservableSensor + StateSensor
  {
    const Lattice l = Lattice::sc(1.0).expand(32, 32, 1).drop_z();
    auto H = hamiltonian(Exchange::from_lattice(1.0, l), Zeeman<IsingSpin>());
    FILE* out = std::tmpfile();
    Machine<decltype(H), GpuIntegrator, IsingSpin>::Instruments ins;
    ins.push_back(std::make_unique<StatSensor<IsingSpin>>(out));
    ins.push_back(std::make_unique<ObservableSensor<IsingSpin>>(dir + "/host_obs.parquet"));
    ins.push_back(std::make_unique<StateSensor<IsingSpin>>(dir + "/host_state.parquet", 7));
    {
      Machine<decltype(H), GpuIntegrator, IsingSpin> m(Thermostat<IsingSpin>(2.8, Field<IsingSpin>::zero()), H,
                                                       MetropolisFlipIntegrator(5), std::move(ins),
                                                       State<IsingSpin>::up_with_size(l.sites_len()));
      check(vg_init_random(m.context()), m.context());
      Relax(20, 4.0).run(m);
      const CoolDown cd(4.0, 1.0, 0.5, 10, 30);
      cd.run(m);
      // the exported state agrees with the device's own totals: |M| of the
      // host copy equals vg_magnetization, and the Compound total of the
      // site energies equals vg_total_energy (integers for Ising, exact)
      const State<IsingSpin> s = m.state();
      double mv[3] = {0, 0, 0}, mag = -1.0;
      check(vg_magnetization(m.context(), mv, &mag), m.context());
      CHECK(std::fabs(s.magnetization().magnitude()) == mag);
      const std::vector<double> es = m.site_energies();
      double sum = 0.0;
      for (double e : es) sum += e;
      CHECK(sum == m.total_energy());
    }
    const std::string stats = slurp(out);
    std::fclose(out);
    CHECK(count_lines(stats) == (int)CoolDown(4.0, 1.0, 0.5).temperatures().size());
    // Parquet files in place of their .parquet.tmp (row counts are checked by
    // the Python test that reads them: relax 20 + 7 x (10 + 30) observable
    // rows; 1024 x (3 + 7 x (2 + 5)) state rows)
    for (const char* f : {"/host_obs.parquet", "/host_state.parquet"}) {
      FILE* p = std::fopen((dir + f).c_str(), "rb");
      CHECK(p != nullptr);
      if (p) {
        const std::string b = slurp(p);
        std::fclose(p);
        CHECK(b.size() > 12 && b.compare(0, 4, "PAR1") == 0 && b.compare(b.size() - 4, 4, "PAR1") == 0);
      }
    }
  }
  // Heisenberg hysteresis with Exchange + Anisotropy + Zeeman
  {
    const Lattice l = Lattice::sc(1.0).expand(8, 8, 8);
    auto H = hamiltonian(Exchange::from_lattice(1.0, l), UniaxialAnisotropy<HeisenbergSpin>(HeisenbergSpin::up(), 0.1),
                         Zeeman<HeisenbergSpin>());
    FILE* out = std::tmpfile();
    Machine<decltype(H), GpuIntegrator, HeisenbergSpin>::Instruments ins;
    ins.push_back(std::make_unique<StatSensor<HeisenbergSpin>>(out));
    Machine<decltype(H), GpuIntegrator, HeisenbergSpin> m(Thermostat<HeisenbergSpin>(1.0, Field<HeisenbergSpin>::zero()), H,
                                                          MetropolisIntegrator(9), std::move(ins),
                                                          State<HeisenbergSpin>::up_with_size(l.sites_len()));
    HysteresisLoop(20, 10, 0.5, 1.0, 0.25).run(m);
    const std::string stats = slurp(out);
    std::fclose(out);
    CHECK(count_lines(stats) == (int)HysteresisLoop(20, 10, 0.5, 1.0, 0.25).fields().size());
    const State<HeisenbergSpin> s = m.state();
    double worst = 0.0;
    for (const auto& v : s.spins()) worst = std::max(worst, std::fabs(std::sqrt(v.dot(v)) - 1.0));
    CHECK(worst < 1e-6);
    // Hamiltonian::energy per site: the Compound total is their sum
    const std::vector<double> e = m.site_energies();
    CHECK(e.size() == l.sites_len());
    double sum = 0.0, mag = 0.0;
    for (double v : e) {
      sum += v;
      mag += std::fabs(v);
    }
    CHECK(std::fabs(sum - m.total_energy()) <= 1e-6 * std::max(1.0, mag));
    CHECK(m.energy(5) == e[5]);
  }
  // Program errors surface before any device work
  {
    const Lattice l = Lattice::sc(1.0).expand(32, 4, 4);
    Machine<Exchange, GpuIntegrator, IsingSpin> m(Thermostat<IsingSpin>(2.0, Field<IsingSpin>::zero()),
                                                  Exchange::from_lattice(1.0, l), MetropolisFlipIntegrator(1), {},
                                                  State<IsingSpin>::up_with_size(l.sites_len()));
    CHECK(throws_program_error([&] { Relax(0, 1.0).run(m); }, ProgramError::Kind::NoSteps));
    CHECK(throws_program_error([&] { Relax(10, 0.0).run(m); }, ProgramError::Kind::ZeroTemperature));
  }
  // The `run` path of the CLI (TOML input -> GPU engine)
  {
    const Input in = Input::parse(
        "model = \"Heisenberg\"\nalgorithm = \"Metropolis\"\nexchange = 1.0\n[sample.unitcell]\nname = \"fcc\"\n"
        "[sample.size]\nx = 4\ny = 4\nz = 4\n[sample.pbc]\nx = true\ny = true\nz = true\n"
        "[[stages]]\nprogram = \"CoolDown\"\nmax_temperature = 2.0\nmin_temperature = 1.0\ncool_rate = 0.5\n"
        "relax = 10\nsteps = 20\n");
    FILE* out = std::tmpfile();
    in.run(3, out);
    CHECK(count_lines(slurp(out)) == 3);
    std::fclose(out);
  }
}

// Rows i = 0..2499 of the observables schema in row groups of 1000:
// relax = i % 3 == 0, stage = i / 100, step = i % 100, n = 100,
// temperature = 1 + i / 1000, field = -0.5 (stored as given), energy = -i / 7,
// magnetization = i * 1e-3.
static void parquet_demo(const std::string& dir) {
  parquet::Writer w(dir + "/demo.parquet", parquet::with_extension(dir + "/demo.parquet", "parquet.tmp"),
                    {{"relax", parquet::Type::Bool},
                     {"stage", parquet::Type::UInt64},
                     {"step", parquet::Type::UInt64},
                     {"n", parquet::Type::UInt64},
                     {"temperature", parquet::Type::Float64},
                     {"field", parquet::Type::Float64},
                     {"energy", parquet::Type::Float64},
                     {"magnetization", parquet::Type::Float64}},
                    1000);
  for (int i = 0; i < 2500; ++i) {
    w.add_bool(0, i % 3 == 0);
    w.add_u64(1, (uint64_t)(i / 100));
    w.add_u64(2, (uint64_t)(i % 100));
    w.add_u64(3, 100);
    w.add_f64(4, 1.0 + i / 1000.0);
    w.add_f64(5, -0.5);
    w.add_f64(6, -i / 7.0);
    w.add_f64(7, i * 1e-3);
    w.end_row();
  }
  w.close();
  CHECK(parquet::with_extension("a/b.parquet", "parquet.tmp") == "a/b.parquet.tmp");
  CHECK(parquet::with_extension("a.d/obs", "parquet.tmp") == "a.d/obs.parquet.tmp");
  CHECK(parquet::with_extension("obs.csv", "parquet.tmp") == "obs.parquet.tmp");
}

int main(int argc, char** argv) {
  const bool cpu = argc > 1 && !std::strcmp(argv[1], "--cpu");
  const bool gpu = argc > 1 && !std::strcmp(argv[1], "--gpu");
  const bool demo = argc > 2 && !std::strcmp(argv[1], "--parquet-demo");
  if (!cpu && !gpu && !demo) {
    std::fprintf(stderr, "usage: %s --cpu | --gpu [DIR] | --parquet-demo DIR\n", argv[0]);
    return 2;
  }
  try {
    if (cpu) cpu_checks();
    if (gpu) gpu_checks(argc > 2 ? argv[2] : ".");
    if (demo) parquet_demo(argv[2]);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAIL exception: %s\n", e.what());
    return 1;
  }
  std::printf("host_selftest %s: %d checks passed\n", cpu ? "cpu" : gpu ? "gpu" : "parquet-demo", g_checks);
  return 0;
}
