/**
 * RandomNumbers.h -- host random numbers for cloud initialisation
 * (RandomNumbers.h:14-32 in the reference: uniform [0,1), uniform [0,2 pi),
 * Gaussian draws from a 64-bit Mersenne Twister).
 *
 * The reference seeds from the clock, so no two runs agree.  Here the seed
 * is RandomNumbers::seed when it is non-zero (the driver's --seed), else a
 * std::random_device draw.  The device thermal force does not use this
 * class: its kicks come from a counter-based generator keyed by
 * ThermalForce's seed.
 */
#ifndef RANDOMNUMBERS
#define RANDOMNUMBERS

#include <cstdint>
#include <random>

class RandomNumbers {
public:
    RandomNumbers();
    ~RandomNumbers() {}
    const double uniformZeroToOne();
    const double uniformZeroToTwoPi();
    const double gaussian(std::normal_distribution<double> &dist);

    static uint64_t seed;  //!< 0: seed from std::random_device

private:
    std::mt19937_64 engine;
    std::uniform_real_distribution<double> zeroToOne;
    std::uniform_real_distribution<double> zeroToTwoPi;
};

#endif  // RANDOMNUMBERS
