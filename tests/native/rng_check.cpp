// Prints the perturbation draws the reference's shape generators make: a default-constructed
// std::default_random_engine feeding uniform_real_distribution<double>(0, eps * dx).
#include <cstdio>
#include <limits>
#include <random>

int main() {
    const double his[3] = {1.0, std::numeric_limits<double>::epsilon() * 0.01, std::numeric_limits<double>::epsilon() * 4e-4};
    for (double hi : his) {
        std::uniform_real_distribution<double> unif(0.0, hi);
        std::default_random_engine re;
        for (int i = 0; i < 12; ++i) std::printf("%.17g\n", unif(re));
    }
    return 0;
}
