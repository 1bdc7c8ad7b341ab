// Shared declarations of the oracle's design-loop helpers (TEST INFRASTRUCTURE ONLY).
#pragma once
#include <cstdint>

extern "C" {
// Counter-based uniform sample in [0,1) keyed by (seed, index).
double orc_uniform(uint64_t seed, uint64_t index);
}
