/* Stand-in for the configuration header that the reference's configure step
 * writes from a template (HEN_HOUSE/pieces/egs_config1.h): the scalar types
 * that the IAEA phase-space library and the egs++ classes built into
 * oracle/_ref take from it, for a 64-bit Linux build with EGS_Float double.
 * The Fortran name-mangling macros are left out: nothing built here calls
 * Fortran. */
#ifndef EGS_CONFIG1_
#define EGS_CONFIG1_
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
