// TEST INFRASTRUCTURE ONLY - runs the reference's own, unmodified
// `Tensor<double>::fastcc_multiply` (contract.hpp:824-912), compiled from the
// reference's sources by oracle/Makefile into oracle/_ref/, so that the tests
// and tests/golden/make_golden.py can pin the oracle restatement to it.
//
// Two accumulator policies are plugged into the reference's template:
//  * RefRecordAcc: TileAccumulator's update semantics (dense T x T tile,
//    first-touch list, `+=` in the reference's loop order,
//    index_tensors.hpp:1028-1037) whose drain records (left index, right
//    index, value) with a correct pos / T, pos % T decode into per-thread
//    vectors. It replaces only the output step that the reference gets wrong.
//  * the shipped TileAccumulator<double> itself, whose ListTensor result is
//    walked to compare its entry count and value multiset.
#include <bitset>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <thread>

#include "contract.hpp"
#include "read.hpp"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <vector>

namespace {

struct Rec {
  std::vector<uint64_t> left, right;
  std::vector<double> val;
};
std::vector<Rec> g_rec;

template <class DT> class RefRecordAcc {
  std::vector<DT> acc;
  std::vector<uint8_t> touched;
  std::vector<uint64_t> first;
  uint64_t L = 0, R = 0, li = 0, ri = 0;

 public:
  RefRecordAcc(uint64_t left_tile_dim, uint64_t right_tile_dim, int)
      : acc(left_tile_dim * right_tile_dim), touched(left_tile_dim * right_tile_dim),
        L(left_tile_dim), R(right_tile_dim) {}
  void reset_accumulator(int i, int j) { li = uint64_t(i); ri = uint64_t(j); }
  void update(uint64_t pos, DT v) {
    if (!touched[pos]) { touched[pos] = 1; first.push_back(pos); }
    acc[pos] += v;
  }
  template <class TensorType, class BCType>
  void drain_into(TensorType &, BCType &, BCType &) {
    Rec &r = g_rec[omp_get_thread_num()];
    for (uint64_t p : first) {
      r.left.push_back(li * L + p / R);
      r.right.push_back(ri * R + p % R);
      r.val.push_back(acc[p]);
      acc[p] = DT();
      touched[p] = 0;
    }
    first.clear();
  }
};

// Field layout of the reference's ListTensor / NNZNode / CompactNNZ /
// CompactCordinate (index_tensors.hpp:13-21,69-126; coordinate.hpp:349-351),
// which offer no accessor for their entries.
struct MirrorCord { int dim; uint32_t *coords; };
struct MirrorNnz { MirrorCord cord; double data; };
struct MirrorNode { MirrorNnz nnz; MirrorNode *next; };
struct MirrorList { MirrorNode *head, *tail; int dim, tid; uint64_t count; };
static_assert(sizeof(MirrorList) == sizeof(ListTensor<double>), "ListTensor layout");

Tensor<double> *make_tensor(int order, int64_t nnz, const int32_t *coords, const double *vals,
                            const int32_t *max_index, std::vector<int> &shape_store) {
  shape_store.assign(max_index, max_index + order);
  // Tensor(int, int, int*) sets `shape` and `dimensionality` (contract.hpp:58-65);
  // its random fill is replaced by the given nonzeros.
  auto *t = new Tensor<double>(0, order, shape_store.data());
  t->delete_old_values();
  auto &nz = t->get_nonzeros();
  nz.reserve(size_t(nnz));
  std::vector<int> sv(shape_store.begin(), shape_store.end());
  for (int64_t n = 0; n < nnz; n++) {
    std::vector<int> c(coords + n * order, coords + (n + 1) * order);
    nz.emplace_back(vals[n], CoOrdinate(c, sv));
  }
  return t;
}

}  // namespace

extern "C" {

// acc_kind 0: RefRecordAcc (correct decode); 1: shipped TileAccumulator<double>.
// Output arrays are malloc'ed; free with ref_free. For acc_kind 1, left/right
// stay NULL and coords holds the (mis-decoded) coordinates the reference emits.
int ref_fastcc_multiply(int32_t ordA, int64_t nnzA, const int32_t *cA, const double *vA,
                        const int32_t *maxA, int32_t ordB, int64_t nnzB, const int32_t *cB,
                        const double *vB, const int32_t *maxB, const int32_t *ctrA,
                        const int32_t *ctrB, int32_t k, int32_t tile_size, int32_t acc_kind,
                        int64_t *n_out, uint64_t **left, uint64_t **right, double **values,
                        int32_t **out_coords, int32_t *out_order, double *ms) {
  if (nnzA < 1 || nnzB < 1) return 1;  // the reference reads nonzeros[0]
  std::vector<int> sa, sb;
  Tensor<double> *a = make_tensor(ordA, nnzA, cA, vA, maxA, sa);
  Tensor<double> *b = make_tensor(ordB, nnzB, cB, vB, maxB, sb);
  CoOrdinate la(std::vector<int>(ctrA, ctrA + k)), lb(std::vector<int>(ctrB, ctrB + k));
  *left = nullptr;
  *right = nullptr;
  *out_coords = nullptr;
  *out_order = ordA + ordB - 2 * k;
  int hc = int(std::thread::hardware_concurrency());
  auto t0 = std::chrono::steady_clock::now();
  if (acc_kind == 0) {
    g_rec.assign(size_t(std::max(hc, 1)), Rec());
    a->fastcc_multiply<RefRecordAcc<double>, double>(*b, la, lb, tile_size);
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    size_t n = 0;
    for (auto &r : g_rec) n += r.val.size();
    *n_out = int64_t(n);
    *left = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    *right = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
    *values = (double *)malloc(sizeof(double) * (n + 1));
    size_t i = 0;
    for (auto &r : g_rec)
      for (size_t q = 0; q < r.val.size(); q++, i++) {
        (*left)[i] = r.left[q];
        (*right)[i] = r.right[q];
        (*values)[i] = r.val[q];
      }
    g_rec.clear();
  } else {
    ListTensor<double> res = a->fastcc_multiply<TileAccumulator<double>, double>(*b, la, lb, tile_size);
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    MirrorList *m = reinterpret_cast<MirrorList *>(&res);
    size_t n = 0;
    for (MirrorNode *p = m->head; p; p = p->next) n++;
    *n_out = int64_t(n);
    *values = (double *)malloc(sizeof(double) * (n + 1));
    *out_coords = (int32_t *)malloc(sizeof(int32_t) * (n * size_t(*out_order) + 1));
    size_t i = 0;
    for (MirrorNode *p = m->head; p; p = p->next, i++) {
      (*values)[i] = p->nnz.data;
      for (int d = 0; d < *out_order; d++) (*out_coords)[i * (*out_order) + d] = int32_t(p->nnz.cord.coords[d]);
    }
  }
  free_heaps();  // the reference's per-call bump heaps (timer.hpp:112-118)
  delete a;
  delete b;
  return 0;
}

// The reference's Tensor<double>::multiply with batch modes
// (contract.hpp:286-367): A's modes batchA[0..nb) are matched with B's
// batchB and kept in the output, ctrA with ctrB are contracted. Its output
// tensor's nonzeros (coordinates: batch, A external, B external) are copied
// to malloc'ed arrays (free with ref_free). Shapes are inferred from the data
// by the reference itself (IndexedTensor calls _infer_shape).
int ref_multiply_modes(int32_t ordA, int64_t nnzA, const int32_t *cA, const double *vA, const int32_t *maxA,
                       int32_t ordB, int64_t nnzB, const int32_t *cB, const double *vB, const int32_t *maxB,
                       const int32_t *ctrA, const int32_t *ctrB, int32_t k, const int32_t *batchA,
                       const int32_t *batchB, int32_t nb, int64_t *n_out, int32_t **out_coords,
                       int32_t *out_order, double **values) {
  if (nnzA < 1 || nnzB < 1) return 1;
  std::vector<int> sa, sb;
  Tensor<double> *a = make_tensor(ordA, nnzA, cA, vA, maxA, sa);
  Tensor<double> *b = make_tensor(ordB, nnzB, cB, vB, maxB, sb);
  CoOrdinate lc(std::vector<int>(ctrA, ctrA + k)), rc(std::vector<int>(ctrB, ctrB + k));
  CoOrdinate lb(std::vector<int>(batchA, batchA + nb)), rb(std::vector<int>(batchB, batchB + nb));
  Tensor<double> res = a->multiply<double, double>(*b, lc, lb, rc, rb);
  auto &nz = res.get_nonzeros();
  const int d = ordA + ordB - 2 * k - nb;
  *out_order = d;
  *n_out = int64_t(nz.size());
  *values = (double *)malloc(sizeof(double) * (nz.size() + 1));
  *out_coords = (int32_t *)malloc(sizeof(int32_t) * (nz.size() * size_t(d) + 1));
  for (size_t i = 0; i < nz.size(); i++) {
    (*values)[i] = nz[i].get_data();
    for (int m = 0; m < d; m++) (*out_coords)[i * d + m] = nz[i].get_coords().get_index(m);
  }
  delete a;
  delete b;
  return 0;
}

void ref_free(void *p) { free(p); }

}  // extern "C"
