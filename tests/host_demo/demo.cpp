// Uses the drop-in header the way the reference's README.md:9-13 and
// benchmark.cpp:44-61 use the reference: read .tns files, infer shapes, call
// fastcc_multiply<TileAccumulator<double>, double>, read the result.
// Usage: demo a.tns b.tns <ctrA: i,j,..> <ctrB: i,j,..> out.txt
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "contract.hpp"
#include "read.hpp"

static std::vector<int> modes(const std::string &s) {
  std::vector<int> m;
  std::stringstream in(s);
  std::string t;
  while (std::getline(in, t, ','))
    if (!t.empty()) m.push_back(std::stoi(t));
  return m;
}

int main(int argc, char **argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s a.tns b.tns ctrA ctrB out.txt\n", argv[0]);
    return 1;
  }
  try {
    Tensor<double> a(argv[1], true), b(argv[2], true);
    a._infer_dimensionality();
    a._infer_shape();
    b._infer_dimensionality();
    b._infer_shape();
    ListTensor<double> r =
        a.fastcc_multiply<TileAccumulator<double>, double>(b, CoOrdinate(modes(argv[3])), CoOrdinate(modes(argv[4])));
    std::FILE *f = std::fopen(argv[5], "w");
    std::fprintf(f, "%d %d\n", r.compute_nnz_count(), r.get_dimensionality());
    for (size_t i = 0; i < r.size(); i++) {
      for (int d = 0; d < r.get_dimensionality(); d++) std::fprintf(f, "%d ", r.coords(i)[d]);
      std::fprintf(f, "%.17g\n", r.value(i));
    }
    std::fclose(f);
    // the README's braced form compiles and runs too
    if (a.get_dimensionality() == 4 && b.get_dimensionality() == 3) {
      ListTensor<double> r2 = a.fastcc_multiply<TileAccumulatorMap<double>, double>(b, {1, 3}, {1, 2});
      if (r2.compute_nnz_count() != r.compute_nnz_count()) return 3;
    }
    // the instrumented twin: five non-negative microsecond figures, [3] the
    // rest of [1] after [2] and [4]
    std::vector<long long> t = a.fastcc_multiply_timing<TileAccumulator<double>, double>(
        b, CoOrdinate(modes(argv[3])), CoOrdinate(modes(argv[4])));
    if (t.size() != 5 || t[0] < 0 || t[1] < 0 || t[2] < 0 || t[4] < 0 || t[3] != t[1] - t[2] - t[4]) return 5;
  } catch (const fcc::Error &e) {
    std::fprintf(stderr, "fcc error %d: %s\n", e.status, e.what());
    return 2;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 4;
  }
  return 0;
}
