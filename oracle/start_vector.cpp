// ORACLE — test infrastructure.  set_random_unit of
// components/linalg_routines/src/lanczos.cpp:55-62: std::mt19937(seed) draws
// std::normal_distribution<double>(0,1) samples, then the vector is normalised.
#include <cmath>
#include <cstdint>
#include <random>

extern "C" void oracle_set_random_unit(double* v, int64_t n, unsigned seed) {
    std::mt19937 rng(seed);
    std::normal_distribution<double> dist(0.0, 1.0);
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        v[i] = dist(rng);
        s += v[i] * v[i];
    }
    s = std::sqrt(s);
    for (int64_t i = 0; i < n; ++i) v[i] /= s;
}
