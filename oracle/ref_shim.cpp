// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C wrappers around the reference's own host helpers, compiled together with
// the reference sources where they lie (ohao/render/rt/env_cdf.cpp,
// sobol_generator.cpp, owen_scramble.cpp) into oracle/_ref/libohao_ref.so by
// `make -C oracle ref`. Used only to pin the oracle's restatement of those
// helpers; the reference tree is read in place, never copied.
#include "render/rt/env_cdf.hpp"
#include "render/rt/sobol_generator.hpp"
#include "render/rt/owen_scramble.hpp"
#include <cstring>

extern "C" {
void ref_env_cdf_build(const float* px, int w, int h, float* marg, float* cond, float* integral) {
    ohao::EnvCDF cdf;
    cdf.build(px, w, h);
    std::memcpy(marg, cdf.marginalCDF().data(), sizeof(float) * static_cast<size_t>(h));
    std::memcpy(cond, cdf.conditionalCDF().data(), sizeof(float) * static_cast<size_t>(w) * static_cast<size_t>(h));
    *integral = cdf.integral();
}
float ref_sobol_sample1d(unsigned index, unsigned dim) { return ohao::SobolGenerator::sample1D(index, dim); }
unsigned ref_owen_scramble(unsigned v, unsigned seed) { return ohao::owenScramble(v, seed); }
const unsigned* ref_sobol_dirs() { return ohao::SobolGenerator::directionNumbers(); }
}
