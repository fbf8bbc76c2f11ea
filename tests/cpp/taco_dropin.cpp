// Drives taco's own API — taco::Tensor<double> statements, TensorBase::compileSource,
// assemble() and compute() (src/tensor.cpp:808-850, 905-930) — with the forwarding source of
// INTEGRATION.md section 2 in place of generated code, for SpMV, SpMM and SpGEMM.
//
// Built against taco's library objects (compiled from the taco sources by
// oracle/Makefile.ref); test infrastructure only.  The forwarding source calls the library's
// taco-ABI entry points (tacogb_<p>_assemble/compute); taco compiles it with TACO_CFLAGS, which
// the caller points at the library to link.  On a machine without a GPU that library is the
// recorder (tests/cpp/tacogb_recorder.c), which writes every argument pack taco passes and
// completes the call with taco's generated code, so that the recorded packs can be replayed
// into libtacogb on a GPU.
//
// Usage: taco_dropin <out_dir>.  For each statement it writes <out_dir>/<p>_expected.bin,
// taco's own result (its default compile path) as the flat arrays of the result tensor, and
// checks that the forwarded result equals it (taco::equals); exit status 0 on success.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "taco.h"

using namespace taco;

namespace {

const char* kForward = R"(
#include "taco_gb300.h"
int assemble(taco_tensor_t* r, taco_tensor_t* a, taco_tensor_t* b) { return tacogb_%s_assemble(r, a, b); }
int compute(taco_tensor_t* r, taco_tensor_t* a, taco_tensor_t* b) { return tacogb_%s_compute(r, a, b); }
)";

std::string forward_source(const char* p) {
  char buf[1024];
  snprintf(buf, sizeof(buf), kForward, p, p);
  return buf;
}

void fill_sparse(Tensor<double>& T, int rows, int cols, double density, unsigned seed) {
  std::mt19937 g(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (int i = 0; i < rows; i++)
    for (int j = 0; j < cols; j++)
      if (u(g) < density) T.insert({i, j}, 2.0 * u(g) - 1.0);
  T.pack();
}

void fill_dense(Tensor<double>& T, std::vector<int> dims, unsigned seed) {
  std::mt19937 g(seed);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  if (dims.size() == 1) {
    for (int i = 0; i < dims[0]; i++) T.insert({i}, u(g));
  } else {
    for (int i = 0; i < dims[0]; i++)
      for (int j = 0; j < dims[1]; j++) T.insert({i, j}, u(g));
  }
  T.pack();
}

// The result's storage as taco holds it: for a CSR result pos, crd and values, for a dense one
// the values.
void dump_result(TensorBase& T, const std::string& path) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { perror(path.c_str()); exit(2); }
  taco_tensor_t* t = T.getTacoTensorT();
  const int order = t->order;
  fwrite(&order, 4, 1, f);
  int64_t count = 1;
  for (int m = 0; m < order; m++) {
    int kind = t->mode_types[m] == taco_mode_sparse ? 1 : 0;
    fwrite(&kind, 4, 1, f);
    if (kind) {
      int32_t* pos = (int32_t*)t->indices[m][0];
      int32_t* crd = (int32_t*)t->indices[m][1];
      const int64_t np = count + 1;
      const int64_t nc = pos[count];
      fwrite(&np, 8, 1, f);
      fwrite(pos, 4, np, f);
      fwrite(&nc, 8, 1, f);
      fwrite(crd, 4, nc, f);
      count = nc;
    } else {
      count *= t->dimensions[m];
    }
  }
  fwrite(&count, 8, 1, f);
  fwrite(t->vals, 8, count, f);
  fclose(f);
}

int check(const char* p, TensorBase& forwarded, TensorBase& expected, const std::string& out) {
  dump_result(expected, out + "/" + p + "_expected.bin");
  if (!equals(forwarded, expected)) {
    fprintf(stderr, "%s: the forwarded result differs from taco's own\n", p);
    return 1;
  }
  printf("%s: forwarded through compileSource, equal to taco's own result\n", p);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: taco_dropin <out_dir>\n");
    return 2;
  }
  const std::string out = argv[1];
  int bad = 0;
  IndexVar i("i"), j("j"), k("k");
  {  // SpMV: y(i) = A(i,j) * x(j), A CSR
    const int n = 301, m = 257;
    Tensor<double> A("A", {n, m}, CSR);
    Tensor<double> x("x", {m}, Format({Dense}));
    fill_sparse(A, n, m, 0.06, 11);
    fill_dense(x, {m}, 12);
    Tensor<double> y("y", {n}, Format({Dense}));
    y(i) = A(i, j) * x(j);
    y.compileSource(forward_source("spmv"));
    y.assemble();
    y.compute();
    Tensor<double> y0("y0", {n}, Format({Dense}));
    y0(i) = A(i, j) * x(j);
    y0.compile();
    y0.assemble();
    y0.compute();
    bad += check("spmv", y, y0, out);
  }
  {  // SpMM: C(i,k) = A(i,j) * B(j,k), A CSR, B and C dense row-major
    const int n = 203, m = 149, N = 24;
    Tensor<double> A("A", {n, m}, CSR);
    Tensor<double> B("B", {m, N}, Format({Dense, Dense}));
    fill_sparse(A, n, m, 0.08, 21);
    fill_dense(B, {m, N}, 22);
    Tensor<double> C("C", {n, N}, Format({Dense, Dense}));
    C(i, k) = A(i, j) * B(j, k);
    C.compileSource(forward_source("spmm"));
    C.assemble();
    C.compute();
    Tensor<double> C0("C0", {n, N}, Format({Dense, Dense}));
    C0(i, k) = A(i, j) * B(j, k);
    C0.compile();
    C0.assemble();
    C0.compute();
    bad += check("spmm", C, C0, out);
  }
  {  // SpGEMM: C(i,k) = A(i,j) * B(j,k), all CSR
    const int n = 181, m = 167, q = 193;
    Tensor<double> A("A", {n, m}, CSR);
    Tensor<double> B("B", {m, q}, CSR);
    fill_sparse(A, n, m, 0.05, 31);
    fill_sparse(B, m, q, 0.05, 32);
    Tensor<double> C("C", {n, q}, CSR);
    C(i, k) = A(i, j) * B(j, k);
    C.compileSource(forward_source("spgemm"));
    C.assemble();
    C.compute();
    Tensor<double> C0("C0", {n, q}, CSR);
    C0(i, k) = A(i, j) * B(j, k);
    C0.compile();
    C0.assemble();
    C0.compute();
    bad += check("spgemm", C, C0, out);
  }
  return bad ? 1 : 0;
}
