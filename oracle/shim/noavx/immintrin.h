// Stand-in for <immintrin.h> on hosts without x86 intrinsics (the aarch64 GPU
// hosts).  The reference's collision source includes it for its AVX2 kernel,
// which is compiled only with -DAVX2, and for the aligned scratch allocation
// of its scalar path (_mm_malloc/_mm_free), the one part a non-AVX2 build
// uses.  Oracle-only test infrastructure: never linked into the product.
#ifndef PLB_ORACLE_SHIM_IMMINTRIN_H_
#define PLB_ORACLE_SHIM_IMMINTRIN_H_
#include "mm_malloc.h"
#endif
