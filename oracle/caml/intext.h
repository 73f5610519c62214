#ifndef ORACLE_CAML_INTEXT_H
#define ORACLE_CAML_INTEXT_H
#include "mlvalues.h"
#define serialize_int_4(x) ((void)(x))
#define serialize_int_8(x) ((void)(x))
#define serialize_block_1(a,b) ((void)(a),(void)(b))
#define serialize_block_4(a,b) ((void)(a),(void)(b))
#define caml_serialize_int_4(x) ((void)(x))
#define caml_serialize_int_8(x) ((void)(x))
#define caml_serialize_block_1(a,b) ((void)(a),(void)(b))
#define caml_serialize_block_4(a,b) ((void)(a),(void)(b))
#define deserialize_uint_4() 0
#define deserialize_sint_4() 0
#define deserialize_uint_8() 0
#define deserialize_sint_8() 0
#define deserialize_block_1(a,b) ((void)(a),(void)(b))
#define deserialize_block_4(a,b) ((void)(a),(void)(b))
#define caml_deserialize_uint_4() 0
#define caml_deserialize_sint_4() 0
#define caml_deserialize_uint_8() 0
#define caml_deserialize_sint_8() 0
#define caml_deserialize_block_1(a,b) ((void)(a),(void)(b))
#define caml_deserialize_block_4(a,b) ((void)(a),(void)(b))
#endif
