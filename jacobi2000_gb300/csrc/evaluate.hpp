// Host helpers of the evaluation path shared by evaluate.cu and roundtrip.cu.
#pragma once

#include "runtime.hpp"

namespace jc {
namespace ev {

// State::add_drop (crates/solvers/src/shallow_water.rs:102-111) on one h plane.
void add_drop(int nx, int ny, float* h, float cx, float cy, float amp, float sigma);
// Normalizer::encode (crates/engine/src/norm.rs:27-34) of planes h, u, v.
void encode(const jc_config& c, const float* h, const float* u, const float* v, long long n, float* out);
// Throws JC_BAD_ARGUMENT unless the drop centre is finite and within 1e6 cells.
void check_centre(float cx, float cy);
// A solver initial state (State::flat + one drop) encoded for the model:
// writes the physical state to `phys` [3][cells] and its encoding to `x`.
void initial_state(const jc_config& c, const jc_drop& d, float* phys, float* x);

}  // namespace ev
}  // namespace jc
