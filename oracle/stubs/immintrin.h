/* Portable stand-in for the three x86 intrinsics the reference's SSSP path
 * uses (_mm_malloc/_mm_free for every array, _rdtsc in utils/timer.c:3-7),
 * so the same recipe builds on x86-64 and AArch64.  _mm_malloc returns
 * zeroed memory.  _rdtsc returns nanoseconds from CLOCK_MONOTONIC (the
 * reference divides by a hard-coded 2.7e9 and only prints the result).
 * Oracle build support, not product code. */
#ifndef GBREF_IMMINTRIN_STUB_H
#define GBREF_IMMINTRIN_STUB_H
#include <stdlib.h>
#include <string.h>
#include <time.h>
static __inline__ void *_mm_malloc(size_t size, size_t align) {
    void *p = NULL;
    if (align < sizeof(void *)) align = sizeof(void *);
    if (posix_memalign(&p, align, size ? size : 1) != 0) return NULL;
    memset(p, 0, size);
    return p;
}
static __inline__ void _mm_free(void *p) { free(p); }
static __inline__ unsigned long long _rdtsc(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (unsigned long long)ts.tv_sec * 1000000000ull + (unsigned long long)ts.tv_nsec;
}
#define _MM_HINT_T0 0
static __inline__ void _mm_prefetch(const char *p, int hint) { (void)p; (void)hint; }
#endif
