#ifndef ORACLE_CAML_BIGARRAY_H
#define ORACLE_CAML_BIGARRAY_H
#include "mlvalues.h"
struct caml_ba_array { void *data; intptr_t num_dims; intptr_t flags; void *proxy; intptr_t dim[3]; };
#define Bigarray_val(v) ((struct caml_ba_array *)(v))
#define Caml_ba_array_val(v) ((struct caml_ba_array *)(v))
#define Data_bigarray_val(v) (Bigarray_val(v)->data)
#define Caml_ba_data_val(v) (Bigarray_val(v)->data)
#define BIGARRAY_INT32 0
#define BIGARRAY_C_LAYOUT 0
#define CAML_BA_INT32 0
#define CAML_BA_C_LAYOUT 0
value oracle_alloc_bigarray(int flags, int ndims, void *data, intptr_t *dims);
#define alloc_bigarray oracle_alloc_bigarray
#define caml_ba_alloc oracle_alloc_bigarray
#define alloc_bigarray_dims(f, n, d, ...) oracle_alloc_bigarray((f), (n), (d), NULL)
#endif
