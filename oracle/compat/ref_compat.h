/* Force-included (gcc -include) when the reference C sources are compiled
 * for the oracle on a non-x86 host.  It gives the handful of x86-only
 * constructs the reference uses the same meaning on aarch64:
 *
 *   __builtin_ia32_maxpd(a, b)  -> per lane (a > b) ? a : b   (SSE2 MAXPD rule:
 *   __builtin_ia32_minpd(a, b)  -> per lane (a < b) ? a : b    the 2nd operand wins
 *                                                               on ties and NaN)
 *   asm "pause"                 -> "yield" (an assembler macro, so the
 *                                  reference's spin loops assemble as-is)
 *
 * Used by approx/step_project.inc, approx/approx.c:272-273 and
 * thread_pool/thread_pool.c:195,222 of the reference.  On x86 hosts this
 * header is not used.
 */
#ifndef ACDALM_REF_COMPAT_H
#define ACDALM_REF_COMPAT_H
#if !defined(__x86_64__) && !defined(__i386__)
typedef double acdalm_compat_v2d __attribute__((vector_size(16)));
static inline acdalm_compat_v2d acdalm_compat_maxpd(acdalm_compat_v2d a,
                                                    acdalm_compat_v2d b)
{
        acdalm_compat_v2d r;
        r[0] = (a[0] > b[0]) ? a[0] : b[0];
        r[1] = (a[1] > b[1]) ? a[1] : b[1];
        return r;
}
static inline acdalm_compat_v2d acdalm_compat_minpd(acdalm_compat_v2d a,
                                                    acdalm_compat_v2d b)
{
        acdalm_compat_v2d r;
        r[0] = (a[0] < b[0]) ? a[0] : b[0];
        r[1] = (a[1] < b[1]) ? a[1] : b[1];
        return r;
}
#define __builtin_ia32_maxpd acdalm_compat_maxpd
#define __builtin_ia32_minpd acdalm_compat_minpd
__asm__(".macro pause\n\tyield\n.endm\n");
#endif
#endif
