/* Stand-in for GCC's x86 header mm_malloc.h, which WDutils' memory.h includes
 * under GCC (usr/dehnen/utils/inc/memory.h:250-252) but which GCC provides on
 * x86 only: _mm_malloc / _mm_free as GCC defines them there, on
 * posix_memalign.  oracle/Makefile puts this directory on the include path
 * only on hosts that are not x86-64. */
#ifndef _MM_MALLOC_H_INCLUDED
#define _MM_MALLOC_H_INCLUDED
#include <stdlib.h>
static inline void *_mm_malloc(size_t size, size_t alignment)
{
    void *p;
    if (alignment == 1) return malloc(size);
    if (alignment == 2 || (sizeof(void *) == 8 && alignment == 4)) alignment = sizeof(void *);
    if (posix_memalign(&p, alignment, size) == 0) return p;
    return (void *)0;
}
static inline void _mm_free(void *p) { free(p); }
#endif
