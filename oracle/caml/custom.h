#ifndef ORACLE_CAML_CUSTOM_H
#define ORACLE_CAML_CUSTOM_H
#include "mlvalues.h"
struct custom_operations {
    char *identifier;
    void (*finalize)(value v);
    int (*compare)(value v1, value v2);
    long (*hash)(value v);
    void (*serialize)(value v, unsigned long *wsize_32, unsigned long *wsize_64);
    unsigned long (*deserialize)(void *dst);
    int (*compare_ext)(value v1, value v2);
};
#define custom_finalize_default NULL
#define custom_compare_default NULL
#define custom_hash_default NULL
#define custom_serialize_default NULL
#define custom_deserialize_default NULL
#define custom_compare_ext_default NULL
value oracle_alloc_custom(struct custom_operations *ops, uintptr_t size, uintptr_t mem, uintptr_t max);
#define alloc_custom oracle_alloc_custom
#define caml_alloc_custom oracle_alloc_custom
#define register_custom_operations(x) ((void)(x))
#define caml_register_custom_operations(x) ((void)(x))
#endif
