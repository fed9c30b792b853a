/* Stand-in for the configuration header that the reference's configure step
 * writes from a template: only the integer types the IAEA phase-space
 * library (HEN_HOUSE/iaea_phsp/iaea_config.h) takes from it. */
#ifndef EGS_CONFIG1_
#define EGS_CONFIG1_
typedef short EGS_I16;
typedef int EGS_I32;
typedef long long EGS_I64;
#endif
