/* The runtime struct taco passes to every generated kernel.  Layout, field meaning and the
 * include guard are those of taco's include/taco/taco_tensor_t.h:11-23, so a translation unit
 * may include both headers and a pointer made by taco (init_taco_tensor_t,
 * src/taco_tensor_t.cpp:32-67, or TensorStorage's conversion, src/storage/storage.cpp:127-177)
 * is passed unchanged to this library.
 *
 *   order          number of modes
 *   dimensions     int32[order]
 *   csize          component size in BITS (64 for double, src/storage/storage.cpp:61-63)
 *   mode_ordering  int32[order]
 *   mode_types     taco_mode_dense / taco_mode_sparse per mode
 *   indices        per mode: dense  -> indices[m][0] is an int32[1] holding the dimension
 *                            sparse -> indices[m][0] = pos (int32[parent+1]),
 *                                      indices[m][1] = crd (int32[nnz])
 *   vals           values
 *   fill_value     csize/8 bytes
 *   vals_size      values array size (unused by generated code)
 */
#ifndef TACO_TENSOR_T_DEFINED
#define TACO_TENSOR_T_DEFINED

#include <stdint.h>

typedef enum { taco_mode_dense, taco_mode_sparse } taco_mode_t;

typedef struct taco_tensor_t {
  int32_t      order;
  int32_t*     dimensions;
  int32_t      csize;
  int32_t*     mode_ordering;
  taco_mode_t* mode_types;
  uint8_t***   indices;
  uint8_t*     vals;
  uint8_t*     fill_value;
  int32_t      vals_size;
} taco_tensor_t;

#endif
