// Stand-in for <mm_malloc.h> on hosts without it (the aarch64 GPU hosts):
// aligned allocation for the reference's scalar collision path.
// Oracle-only test infrastructure: never linked into the product.
#ifndef PLB_ORACLE_SHIM_MM_MALLOC_H_
#define PLB_ORACLE_SHIM_MM_MALLOC_H_
#include <stdlib.h>

static inline void* _mm_malloc(size_t size, size_t align) {
    void* p = NULL;
    if (align < sizeof(void*)) align = sizeof(void*);
    return posix_memalign(&p, align, size) == 0 ? p : NULL;
}
static inline void _mm_free(void* p) { free(p); }
#endif
