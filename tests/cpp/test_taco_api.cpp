// taco's API over libtacogb: the known-answer and randomized tests of taco's own suite for the
// three statements, written as a taco user writes them.  Exit status 0 = all passed.
//   expr_storage spmv  (test/tests-expr_storage.cpp:873-937): d33a * d3b = {0,0,18}
//   expr_storage matrix_mul (:996-1035): d33a * d33b = {0,0,0, 0,0,0, 30,180,0}
//   scheduling_eval spmvCPU / spmmCPU / spgemm (test/tests-scheduling-eval.cpp:549-662,
//   843-889): srand(75883) inputs, compared with the same statement evaluated by plain loops.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "taco_gb300/taco.hpp"

using namespace taco;

static int failures = 0;
#define EXPECT(cond, ...)                                  \
  do {                                                     \
    if (!(cond)) {                                         \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__);     \
      std::printf(__VA_ARGS__);                            \
      std::printf("\n");                                   \
      failures++;                                          \
    }                                                      \
  } while (0)

static void test_spmv_kat() {
  Tensor<double> B("B", {3, 3}, Format({Dense, Sparse}));
  B.insert({0, 1}, 2); B.insert({2, 0}, 3); B.insert({2, 2}, 4); B.pack();
  Tensor<double> c("c", {3}, Format({Dense}));
  c.insert({0}, 2); c.insert({2}, 3); c.pack();
  Tensor<double> a("a", {3}, Format({Dense}));
  IndexVar i, k;
  a(i) = B(i, k) * c(k);
  a.compile(); a.assemble(); a.compute();
  EXPECT(a.at({0}) == 0 && a.at({1}) == 0 && a.at({2}) == 18, "spmv KAT got %g %g %g",
         a.at({0}), a.at({1}), a.at({2}));
}

static void test_matmul_kat() {
  Tensor<double> B("B", {3, 3}, CSR);
  B.insert({0, 1}, 2); B.insert({2, 0}, 3); B.insert({2, 2}, 4); B.pack();
  Tensor<double> Cd("C", {3, 3}, Format({Dense, Dense}));
  Cd.insert({0, 0}, 10); Cd.insert({0, 1}, 20); Cd.insert({2, 1}, 30); Cd.pack();
  Tensor<double> a("a", {3, 3}, Format({Dense, Dense}));
  IndexVar i, j, k;
  a(i, j) = B(i, k) * Cd(k, j);
  a.evaluate();
  const double want[9] = {0, 0, 0, 0, 0, 0, 30, 180, 0};
  for (int q = 0; q < 9; q++) EXPECT(a.at({q / 3, q % 3}) == want[q], "matmul dense [%d]", q);
  // the same product with a CSR right operand and a CSR result (SpGEMM)
  Tensor<double> Cs("Cs", {3, 3}, CSR);
  Cs.insert({0, 0}, 10); Cs.insert({0, 1}, 20); Cs.insert({2, 1}, 30); Cs.pack();
  Tensor<double> s("s", {3, 3}, CSR);
  s(i, j) = B(i, k) * Cs(k, j);
  s.evaluate();
  EXPECT(s.nnz() == 2 && s.at({2, 0}) == 30 && s.at({2, 1}) == 180, "matmul CSR nnz %lld",
         (long long)s.nnz());
}

// Fill as taco's randomized tests do: rand_float = (float)rand()/(float)RAND_MAX; insert when
// rand_float < SPARSITY with value (double)(int)(rand_float*3/SPARSITY).
template <typename T>
static void fill_random(Tensor<T>& t, float sparsity, bool sparse) {
  const auto& d = t.getDimensions();
  for (int i = 0; i < d[0]; i++)
    for (int j = 0; j < d[1]; j++) {
      float r = (float)rand() / (float)(RAND_MAX);
      if (!sparse || r < sparsity) t.insert({i, j}, (T)((int)(r * 3 / sparsity)));
    }
  t.pack();
}

static void test_spmv_random() {
  const int NI = 1021 / 10, NJ = 1039 / 10;
  const float SP = .3f;
  Tensor<double> A("A", {NI, NJ}, CSR);
  Tensor<double> x("x", {NJ}, Format({Dense}));
  Tensor<double> y("y", {NI}, Format({Dense}));
  srand(120);
  fill_random(A, SP, true);
  std::vector<double> xv(NJ);
  for (int j = 0; j < NJ; j++) {
    xv[j] = (double)((int)((float)rand() / (float)(RAND_MAX) * 3 / SP));
    x.insert({j}, xv[j]);
  }
  x.pack();
  IndexVar i, j;
  y(i) = A(i, j) * x(j);
  y.compile(); y.assemble(); y.compute();
  for (int r = 0; r < NI; r++) {
    double e = 0;
    for (int32_t q = A.pos()[r]; q < A.pos()[r + 1]; q++) e += A.vals()[q] * xv[A.crd()[q]];
    EXPECT(std::fabs(y.at({r}) - e) <= 1e-12 * std::fabs(e), "spmv row %d: %g vs %g", r, y.at({r}), e);
  }
}

static void test_spmm_random() {
  const int NI = 1021 / 10, NJ = 1039 / 10, NK = 128;
  const float SP = .3f;
  Tensor<double> A("A", {NI, NJ}, CSR);
  Tensor<double> B("B", {NJ, NK}, Format({Dense, Dense}));
  Tensor<double> C("C", {NI, NK}, Format({Dense, Dense}));
  srand(75883);
  fill_random(A, SP, true);
  fill_random(B, SP, false);
  IndexVar i, j, k;
  C(i, k) = A(i, j) * B(j, k);
  C.compile(); C.assemble(); C.compute();
  for (int r = 0; r < NI; r++)
    for (int c = 0; c < NK; c++) {
      double e = 0;
      for (int32_t q = A.pos()[r]; q < A.pos()[r + 1]; q++) e += A.vals()[q] * B.at({A.crd()[q], c});
      EXPECT(std::fabs(C.at({r, c}) - e) <= 1e-12 * std::fabs(e), "spmm (%d,%d)", r, c);
    }
}

static void test_spgemm_random() {
  const int N = 100;
  const float SP = .03f;
  Tensor<double> A("A", {N, N}, CSR);
  Tensor<double> B("B", {N, N}, CSR);
  Tensor<double> C("C", {N, N}, CSR);
  srand(75883);
  fill_random(A, SP, true);
  fill_random(B, SP, true);
  IndexVar i, j, k;
  C(i, k) = A(i, j) * B(j, k);
  C.compile(); C.assemble(); C.compute();
  // expected by a dense workspace per row (taco's default lowering)
  int64_t nnz = 0;
  for (int r = 0; r < N; r++) {
    std::vector<double> w(N, 0.0);
    std::vector<char> set(N, 0);
    for (int32_t p = A.pos()[r]; p < A.pos()[r + 1]; p++) {
      const int j2 = A.crd()[p];
      for (int32_t q = B.pos()[j2]; q < B.pos()[j2 + 1]; q++) {
        w[B.crd()[q]] += A.vals()[p] * B.vals()[q];
        set[B.crd()[q]] = 1;
      }
    }
    int32_t t = C.pos()[r];
    for (int c = 0; c < N; c++) {
      if (!set[c]) continue;
      EXPECT(t < C.pos()[r + 1] && C.crd()[t] == c, "spgemm crd row %d col %d", r, c);
      EXPECT(C.vals()[t] == w[c], "spgemm value (%d,%d)", r, c);
      t++;
      nnz++;
    }
    EXPECT(t == C.pos()[r + 1], "spgemm row %d length", r);
  }
  EXPECT(nnz == C.nnz(), "spgemm nnz %lld vs %lld", (long long)nnz, (long long)C.nnz());
}

static void test_unsupported_throws() {
  Tensor<double> A("A", {4, 4}, Format({Dense, Dense}));
  Tensor<double> x("x", {4}, Format({Dense}));
  Tensor<double> y("y", {4}, Format({Dense}));
  A.pack(); x.pack();
  IndexVar i, j;
  y(i) = A(i, j) * x(j);
  bool threw = false;
  try {
    y.compile();
  } catch (const std::runtime_error&) {
    threw = true;
  }
  EXPECT(threw, "dense A must be refused (taco generates code for it)");
}

int main() {
  test_spmv_kat();
  test_matmul_kat();
  test_spmv_random();
  test_spmm_random();
  test_spgemm_random();
  test_unsupported_throws();
  std::printf(failures ? "%d failures\n" : "all passed\n", failures);
  return failures ? 1 : 0;
}
