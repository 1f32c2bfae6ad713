// Determinism shim for building the reference sources as a test oracle (TEST INFRASTRUCTURE ONLY).
//
// The reference seeds its generators from std::random_device (src/crt/do_render.hpp:49,
// src/crt/materials/material.hpp:98,122,148, src/crt/lights/area_light.hpp:19).  This header is
// force-included (g++ -include) ahead of the reference sources: it pulls in <random> first and then
// renames every later use of `random_device` to a counter-based stand-in, so two runs of the oracle
// build draw the same sequence.  The reference sources themselves are not modified.
#pragma once
#include <random>
#include <cstdint>

namespace crt_ref_shim {
struct counter_device {
    using result_type = unsigned int;
    static unsigned int& counter() {
        static unsigned int c = 0x1234567u;
        return c;
    }
    counter_device() = default;
    explicit counter_device(const std::string&) {}
    unsigned int operator()() {
        unsigned int x = (counter() += 0x9E3779B9u);
        x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
        return x;
    }
    static constexpr unsigned int min() { return 0u; }
    static constexpr unsigned int max() { return 0xffffffffu; }
    double entropy() const noexcept { return 0.0; }
};
}  // namespace crt_ref_shim

namespace std {
using crt_ref_counter_device = ::crt_ref_shim::counter_device;
}
#define random_device crt_ref_counter_device
