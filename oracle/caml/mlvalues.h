/* Minimal stand-in for the OCaml runtime headers, written for this project so
 * that the reference's C kernels can be compiled and called from plain C test
 * drivers.  Values are untagged machine words; custom blocks are raw pointers.
 * This file is test infrastructure: nothing in the shipped library uses it. */
#ifndef ORACLE_CAML_STUB_H
#define ORACLE_CAML_STUB_H
#include <stdint.h>
#include <stdlib.h>
#include <stdio.h>
typedef intptr_t value;
typedef int32_t int32;
typedef uint32_t uint32;
typedef int64_t int64;
typedef uintptr_t mlsize_t;
typedef unsigned int tag_t;
#define Val_int(x) ((value)(x))
#define Int_val(x) ((int)(x))
#define Val_long(x) ((value)(x))
#define Long_val(x) ((long)(x))
#define Unsigned_long_val(x) ((unsigned long)(x))
#define Val_bool(x) ((value)((x) != 0))
#define Bool_val(x) ((int)((x) != 0))
#define Val_true ((value)1)
#define Val_false ((value)0)
#define Val_unit ((value)0)
#define Val_emptylist ((value)0)
#define Data_custom_val(v) ((void *)(v))
#define Field(v, i) (((value *)(v))[i])
#define Store_field(b, i, v) (Field(b, i) = (v))
#define Double_val(v) (*(double *)(v))
#define Int32_val(v) (*(int32_t *)(v))
#define Int64_val(v) (*(int64_t *)(v))
#define Wosize_val(v) ((mlsize_t)0)
#define Is_block(v) ((v) != 0)
#define Tag_val(v) 0
#define CAMLparam0()
#define CAMLparam1(a) (void)(a)
#define CAMLparam2(a,b) (void)(a);(void)(b)
#define CAMLparam3(a,b,c) (void)(a);(void)(b);(void)(c)
#define CAMLparam4(a,b,c,d) (void)(a);(void)(b);(void)(c);(void)(d)
#define CAMLparam5(a,b,c,d,e) (void)(a);(void)(b);(void)(c);(void)(d);(void)(e)
#define CAMLxparam1(a) (void)(a)
#define CAMLxparam2(a,b) (void)(a);(void)(b)
#define CAMLxparam3(a,b,c) (void)(a);(void)(b);(void)(c)
#define CAMLxparam4(a,b,c,d) (void)(a);(void)(b);(void)(c);(void)(d)
#define CAMLxparam5(a,b,c,d,e) (void)(a);(void)(b);(void)(c);(void)(d);(void)(e)
#define CAMLlocal1(a) value a = 0
#define CAMLlocal2(a,b) value a = 0, b = 0
#define CAMLlocal3(a,b,c) value a = 0, b = 0, c = 0
#define CAMLlocal4(a,b,c,d) value a = 0, b = 0, c = 0, d = 0
#define CAMLlocal5(a,b,c,d,e) value a = 0, b = 0, c = 0, d = 0, e = 0
#define CAMLreturn(x) return (x)
#define CAMLreturn0 return
#define CAMLreturnT(t, x) return (x)
#define CAMLprim
#define CAMLextern extern
#endif
