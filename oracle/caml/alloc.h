#ifndef ORACLE_CAML_ALLOC_H
#define ORACLE_CAML_ALLOC_H
#include "mlvalues.h"
value oracle_copy_double(double d);
value oracle_alloc(uintptr_t n, int tag);
#define caml_copy_double oracle_copy_double
#define copy_double oracle_copy_double
#define caml_alloc oracle_alloc
#define alloc oracle_alloc
#define alloc_tuple(n) oracle_alloc((n), 0)
#define caml_alloc_tuple(n) oracle_alloc((n), 0)
#define alloc_small oracle_alloc
#define caml_alloc_small oracle_alloc
#endif
