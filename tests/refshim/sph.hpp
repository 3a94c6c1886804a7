// sph.hpp (tests only) -- stands in for the reference's hydrocodes/sph/sph.hpp so
// that the reference's own drivers (cpu_dump.cpp, cpu_bench.cpp, which include
// "sph.hpp") compile unchanged against the GPU library's System facade and link
// against libdeorbit_sph.so.  The standard headers are the ones the reference
// header brings in and its drivers rely on (std::max, std::mt19937, ...).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <thread>
#include <vector>

#include "deorbit_sph_system.hpp"
