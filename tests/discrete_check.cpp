// Prints, for a seed and a weight vector, the uniforms that
// std::uniform_real_distribution<double>(0,1) draws from std::mt19937_64 and
// the outcomes std::discrete_distribution draws from a second engine with the
// same seed (RngEngine::rand(0,1) and RngEngine::rand_int(probs) of the
// reference, framework/rng.hpp), one pair per line.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

int main(int argc, char **argv) {
  const unsigned long long seed = std::strtoull(argv[1], nullptr, 10);
  const int draws = std::atoi(argv[2]);
  std::vector<double> w;
  for (int i = 3; i < argc; ++i) w.push_back(std::strtod(argv[i], nullptr));
  std::mt19937_64 a(seed), b(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (int i = 0; i < draws; ++i) {
    const double x = u(a);
    const size_t k = std::discrete_distribution<size_t>(w.begin(), w.end())(b);
    std::printf("%.17g %zu\n", x, k);
  }
  return 0;
}
