/**
 * RandomNumbers.cpp -- seeded 64-bit Mersenne Twister draws.
 */
#include "RandomNumbers.h"

#include <cmath>

uint64_t RandomNumbers::seed = 0;

namespace {
uint64_t first_seed() {
    if (RandomNumbers::seed) return RandomNumbers::seed;
    std::random_device rd;
    return ((uint64_t)rd() << 32) ^ (uint64_t)rd();
}
}  // namespace

RandomNumbers::RandomNumbers() : engine(first_seed()), zeroToOne(0.0, 1.0), zeroToTwoPi(0.0, 2.0 * M_PI) {}

const double RandomNumbers::uniformZeroToOne() { return zeroToOne(engine); }
const double RandomNumbers::uniformZeroToTwoPi() { return zeroToTwoPi(engine); }
const double RandomNumbers::gaussian(std::normal_distribution<double> &dist) { return dist(engine); }
