/* Stand-in for <xmmintrin.h> on non-x86 hosts, used only when compiling the
 * reference sources for the oracle.  The reference includes it for
 * _mm_prefetch, which it calls only when PREFETCH_DISTANCE != 0 (it is 0 by
 * default), so a no-op prefetch keeps its meaning. */
#ifndef ACDALM_COMPAT_XMMINTRIN_H
#define ACDALM_COMPAT_XMMINTRIN_H
#define _MM_HINT_NTA 0
#define _mm_prefetch(p, hint) ((void)(p), (void)(hint))
#endif
