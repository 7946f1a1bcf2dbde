// vegas.hpp -- C++ host mirror of the vegas crate's hot-path API on top of
// the GB300 engine (libvegas_gpu, include/vegas_gpu.h).  Module map, after
// src/lib.rs:127-140:
//   accumulator.hpp  src/accumulator.rs
//   energy.hpp       src/energy.rs
//   error.hpp        src/error.rs
//   input.hpp        src/input.rs
//   instrument.hpp   src/instrument.rs (+ the output schemas of src/output.rs)
//   lattice.hpp      the vegas-lattice calls the reference makes
//   machine.hpp      src/machine.rs, src/integrator.rs (GPU integrators)
//   program.hpp      src/program.rs
//   state.hpp        src/state.rs
//   thermostat.hpp   src/thermostat.rs
#pragma once

#include "accumulator.hpp"
#include "energy.hpp"
#include "error.hpp"
#include "input.hpp"
#include "instrument.hpp"
#include "lattice.hpp"
#include "machine.hpp"
#include "program.hpp"
#include "snappy.hpp"
#include "state.hpp"
#include "thermostat.hpp"
