// Test-infrastructure driver: runs the reference's own parallel_sample
// (src/fri_utils.cpp:176-362, compiled from its sources by `make -C oracle
// ref`) on one probability vector and prints what it returns.
//
//   ref_parallel_sample <q.bin> <n_sample> <threads> <seed>
//
// q.bin holds the float64 vector.  srand(seed) precedes the call, with
// omp_set_num_threads(threads) (the reference's number of chunks).  Output:
// one line with the sampled indices, then one line with the next four rand()
// values (the caller finds how many draws the call consumed from them).
#include <omp.h>

#include <cstdio>
#include <cstdlib>
#include <span>
#include <vector>

#include <fri_utils.hpp>

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::vector<double> q;
  double v;
  while (std::fread(&v, sizeof(double), 1, f) == 1) q.push_back(v);
  std::fclose(f);
  const size_t n_sample = std::strtoull(argv[2], nullptr, 10);
  omp_set_num_threads(std::atoi(argv[3]));
  srand((unsigned)std::strtoul(argv[4], nullptr, 10));
  std::vector<size_t> S = parallel_sample(n_sample, std::span<double const>(q.data(), q.size()));
  for (size_t k = 0; k < S.size(); ++k) std::printf(k ? " %zu" : "%zu", S[k]);
  std::printf("\n");
  for (int k = 0; k < 4; ++k) std::printf(k ? " %d" : "%d", rand());
  std::printf("\n");
  return 0;
}
