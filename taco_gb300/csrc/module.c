/* Per-pattern drop-in module.  Compiled once per statement with -DTACOGB_PATTERN=<p>, it
 * exports exactly the symbols a taco-compiled kernel module exports — assemble, compute,
 * evaluate and their packed _shim_ forms (src/codegen/codegen_c.cpp:591-630,
 * src/codegen/codegen_cuda.cpp:1500-1540) — so that ir::Module's dlopen/dlsym path
 * (src/codegen/module.cpp:163-180) or a compileSource user can load it in place of the JIT'd
 * object.  Each symbol forwards to the prefixed entry point in libtacogb.
 */
#include "taco_gb300.h"

#ifndef TACOGB_PATTERN
#error "define TACOGB_PATTERN (spmv, spmm, spgemm, sddmm, ttv, ttm or mttkrp)"
#endif
/* tensors per call: 3 (result and two operands), 4 for sddmm and mttkrp (A, B, C, D) */
#ifndef TACOGB_NARGS
#define TACOGB_NARGS 3
#endif

#define TACOGB_CAT_(a, b, c) a##b##c
#define TACOGB_CAT(a, b, c) TACOGB_CAT_(a, b, c)
#define TACOGB_FN(name) TACOGB_CAT(tacogb_, TACOGB_PATTERN, _##name)
#define TACOGB_SHIM(name) TACOGB_CAT(_shim_tacogb_, TACOGB_PATTERN, _##name)

#if TACOGB_NARGS == 4
int assemble(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b, taco_tensor_t* c) { return TACOGB_FN(assemble)(out, a, b, c); }
int compute(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b, taco_tensor_t* c) { return TACOGB_FN(compute)(out, a, b, c); }
int evaluate(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b, taco_tensor_t* c) { return TACOGB_FN(evaluate)(out, a, b, c); }
#else
int assemble(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b) { return TACOGB_FN(assemble)(out, a, b); }
int compute(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b) { return TACOGB_FN(compute)(out, a, b); }
int evaluate(taco_tensor_t* out, taco_tensor_t* a, taco_tensor_t* b) { return TACOGB_FN(evaluate)(out, a, b); }
#endif
int _shim_assemble(void** args) { return TACOGB_SHIM(assemble)(args); }
int _shim_compute(void** args) { return TACOGB_SHIM(compute)(args); }
int _shim_evaluate(void** args) { return TACOGB_SHIM(evaluate)(args); }
