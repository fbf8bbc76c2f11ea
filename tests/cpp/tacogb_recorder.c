/* A stand-in for libtacogb that records the taco-ABI calls taco makes into it (test
 * infrastructure only, for a machine without a GPU).  It exports tacogb_<p>_assemble and
 * tacogb_<p>_compute for p in spmv, spmm, spgemm with the library's signatures
 * (include/taco_gb300.h); each call appends its argument pack — for every tensor its order,
 * csize, dimensions, mode ordering and mode types, and the index arrays and values it holds — to
 * $TACOGB_RECORD_DIR/<p>_<fn>.bin, then completes the call with taco's own generated code for the
 * statement ($TACOGB_REF_DIR/libtacoref_<p>.so, built by oracle/Makefile.ref), as the module
 * taco would otherwise have compiled.  tests/golden/make_golden.py turns the records into the
 * fixtures that tests/test_taco_dropin_gpu.py replays into libtacogb on a GPU. */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "taco_gb300_tensor.h"

typedef int (*kernel_fn)(taco_tensor_t*, taco_tensor_t*, taco_tensor_t*);

static void put(FILE* f, const void* p, size_t bytes) {
  if (bytes && fwrite(p, 1, bytes, f) != bytes) {
    perror("recorder");
    exit(3);
  }
}

static void put_i64(FILE* f, int64_t v) { put(f, &v, 8); }

/* One tensor: header, then per mode its arrays (sparse: pos and crd when present), then values
 * (when present).  Array lengths follow from the levels above, as taco derives them.  A result
 * before assembly holds no arrays yet (whatever its pointers say): header only. */
static void record_tensor(FILE* f, const taco_tensor_t* t, int header_only) {
  put_i64(f, t->order);
  put_i64(f, t->csize);
  for (int m = 0; m < t->order; m++) put_i64(f, t->dimensions[m]);
  for (int m = 0; m < t->order; m++) put_i64(f, t->mode_ordering ? t->mode_ordering[m] : m);
  for (int m = 0; m < t->order; m++) put_i64(f, t->mode_types[m]);
  int64_t count = 1;
  int complete = !header_only;
  for (int m = 0; m < t->order; m++) {
    if (t->mode_types[m] == taco_mode_dense) {
      count *= t->dimensions[m];
      continue;
    }
    const int32_t* pos = t->indices && t->indices[m] ? (const int32_t*)t->indices[m][0] : NULL;
    const int32_t* crd = t->indices && t->indices[m] ? (const int32_t*)t->indices[m][1] : NULL;
    if (!complete || !pos || !crd) {
      put_i64(f, -1);  /* not assembled yet */
      complete = 0;
      continue;
    }
    const int64_t np = count + 1, nc = pos[count];
    put_i64(f, np);
    put(f, pos, 4 * (size_t)np);
    put_i64(f, nc);
    put(f, crd, 4 * (size_t)nc);
    count = nc;
  }
  if (complete && t->vals) {
    put_i64(f, count);
    put(f, t->vals, (size_t)count * (size_t)(t->csize / 8));
  } else {
    put_i64(f, -1);
  }
}

static int record_and_run(const char* pattern, const char* fn, taco_tensor_t* r,
                          taco_tensor_t* a, taco_tensor_t* b) {
  const char* dir = getenv("TACOGB_RECORD_DIR");
  const char* ref = getenv("TACOGB_REF_DIR");
  if (!dir || !ref) {
    fprintf(stderr, "recorder: set TACOGB_RECORD_DIR and TACOGB_REF_DIR\n");
    return 1;
  }
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s_%s.bin", dir, pattern, fn);
  FILE* f = fopen(path, "ab");
  if (!f) {
    perror(path);
    return 1;
  }
  put_i64(f, 3);
  record_tensor(f, r, strcmp(fn, "assemble") == 0);
  record_tensor(f, a, 0);
  record_tensor(f, b, 0);
  fclose(f);
  snprintf(path, sizeof(path), "%s/libtacoref_%s.so", ref, pattern);
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    fprintf(stderr, "recorder: %s\n", dlerror());
    return 1;
  }
  kernel_fn k = (kernel_fn)dlsym(h, fn);
  return k ? k(r, a, b) : 1;
}

#define RECORDED(p)                                                                      \
  int tacogb_##p##_assemble(taco_tensor_t* r, taco_tensor_t* a, taco_tensor_t* b) {    \
    return record_and_run(#p, "assemble", r, a, b);                                      \
  }                                                                                      \
  int tacogb_##p##_compute(taco_tensor_t* r, taco_tensor_t* a, taco_tensor_t* b) {     \
    return record_and_run(#p, "compute", r, a, b);                                       \
  }

RECORDED(spmv)
RECORDED(spmm)
RECORDED(spgemm)
