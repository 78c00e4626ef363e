// fcc_benchmark - command-line benchmark of the GB300 contraction, with the
// arguments and report of the reference's benchmark driver (benchmark.cpp:9-121
// of jianjianh1/fastcc-benchmark):
//
//   fcc_benchmark <tensor.tns> <modes: m1,m2,...> [tile_size = 128] [dense: 0|1]
//
// It reads a FROSTT .tns file (first line a header), contracts the tensor with
// itself over the given modes (the same list on both sides), three times with
// fastcc_multiply_timing and three times with a wall-clocked fastcc_multiply,
// and prints the median of each figure in microseconds. `dense` picks the
// accumulator tag (TileAccumulator / TileAccumulatorMap); on the GPU both give
// the same result. The reference labels figures [3] and [4] of its timing
// vector "Drain" and "Indexing" in the wrong order (benchmark.cpp:118-119
// against contract.hpp:809-814); here each figure carries its own name.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "contract.hpp"
#include "read.hpp"

namespace {

std::vector<int> parse_modes(const std::string &s) {
  std::vector<int> out;
  size_t i = 0;
  while (i <= s.size()) {
    size_t j = s.find(',', i);
    if (j == std::string::npos) j = s.size();
    if (j > i) out.push_back(std::stoi(s.substr(i, j - i)));
    i = j + 1;
  }
  return out;
}

long long median(std::vector<long long> v) {
  std::sort(v.begin(), v.end());
  return v[v.size() / 2];
}

template <class Acc>
void run(Tensor<double> &t, const CoOrdinate &modes, int tile, int iters,
         std::vector<std::vector<long long>> &fig) {
  for (int it = 0; it < iters; it++) {
    std::vector<long long> f = t.fastcc_multiply_timing<Acc, double, double>(t, modes, modes, tile);
    const auto t0 = std::chrono::steady_clock::now();
    ListTensor<double> r = t.fastcc_multiply<Acc, double, double>(t, modes, modes, tile);
    const auto t1 = std::chrono::steady_clock::now();
    f.push_back(std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count());
    for (size_t k = 0; k < f.size(); k++) fig[k].push_back(f[k]);
    std::printf("run %d: %d nonzeros\n", it, r.compute_nnz_count());
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) {
    std::printf("Usage: %s <tensor_file> <mode: i_1,i_2,...> [tile_size] [dense: 0|1]\n", argv[0]);
    return 1;
  }
  const int tile = argc > 3 ? std::atoi(argv[3]) : 128;
  const bool dense = argc > 4 && std::atoi(argv[4]) != 0;
  try {
    std::printf("Loading tensor...\n");
    Tensor<double> t(argv[1], true);
    std::printf("Loaded tensor.\n");
    t._infer_dimensionality();
    t._infer_shape();
    const CoOrdinate modes(parse_modes(argv[2]));
    std::vector<std::vector<long long>> fig(6);
    if (dense)
      run<TileAccumulator<double>>(t, modes, tile, 3, fig);
    else
      run<TileAccumulatorMap<double>>(t, modes, tile, 3, fig);
    const char *names[6] = {"Index build", "Compute", "Drain", "Accumulate", "Indexing", "Total"};
    for (int k = 0; k < 6; k++) std::printf("%s time: %lld us\n", names[k], median(fig[k]));
  } catch (const fcc::Error &e) {
    std::fprintf(stderr, "fcc error %d: %s\n", e.status, e.what());
    return 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 3;
  }
  return 0;
}
