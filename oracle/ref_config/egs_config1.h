/* Stand-in for the configuration header that the reference's configure step
 * writes from a template (HEN_HOUSE/pieces/egs_config1.h): the scalar types
 * that the IAEA phase-space library and the egs++ classes built into
 * oracle/_ref take from it, for a 64-bit Linux build with EGS_Float double,
 * and the Fortran name mangling of gfortran (one trailing underscore), with
 * which the egs++ application interface declares its Fortran entry points. */
#ifndef EGS_CONFIG1_
#define EGS_CONFIG1_
#define F77_OBJ(fname, FNAME) fname##_
#define F77_OBJ_(fname, FNAME) fname##_
#define CONFIG_NAME "oracle_ref"
#ifdef __cplusplus
#define __extc__ "C"
#else
#define __extc__
#endif
typedef double EGS_Float;
typedef short EGS_I16;
typedef int EGS_I32;
typedef long long EGS_I64;
#endif
