#ifndef ORACLE_CAML_FAIL_H
#define ORACLE_CAML_FAIL_H
#include "mlvalues.h"
static inline void oracle_failwith(const char *m) { fprintf(stderr, "failwith: %s\n", m); abort(); }
#define failwith(m) oracle_failwith(m)
#define caml_failwith(m) oracle_failwith(m)
#define invalid_argument(m) oracle_failwith(m)
#define caml_invalid_argument(m) oracle_failwith(m)
#endif
