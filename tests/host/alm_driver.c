/* The reference's TEST_ALM driver (alm.c:366-395) as a caller would keep
 * it after switching to libacdalm: plain C against include/alm.h, linked
 * with -lacdalm instead of the reference's objects.  Reads an instance in
 * alm_read's text format, solves it, prints the return value, c'x and the
 * largest |A x - b|; a device failure prints acdalm_last_error() and exits
 * with status 2. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "acdalm_ext.h"
#include "alm.h"

int main(int argc, char ** argv)
{
        if (argc < 2)
                return 3;
        sparse_matrix_init();
        FILE * f = fopen(argv[1], "r");
        if (!f)
                return 3;
        alm_t * alm = alm_read(f);
        fclose(f);
        if (!alm)
                return 3;
        size_t n = alm_nvars(alm), m = alm_nrhs(alm);
        double * x = calloc(n, sizeof(double));
        double * y = calloc(m, sizeof(double));
        int r = alm_solve(alm, 1000, x, n, y, m, NULL, NULL, NULL);
        if (r < 0) {
                fprintf(stderr, "alm_solve: %d: %s\n", r, acdalm_last_error());
                return 2;
        }
        const double * c = alm_linear(alm);
        double cx = 0;
        for (size_t j = 0; j < n; j++)
                cx += c[j] * x[j];
        double * ax = calloc(m, sizeof(double));
        sparse_matrix_multiply(ax, m, alm_matrix(alm), x, n, 0, NULL);
        const double * b = alm_rhs(alm);
        double viol = 0;
        for (size_t i = 0; i < m; i++)
                viol = fmax(viol, fabs(ax[i] - b[i]));
        printf("ret %d objective %.12g max_violation %.3g\n", r, cx, viol);
        sparse_matrix_free(alm_matrix(alm));
        alm_free(alm);
        free(x);
        free(y);
        free(ax);
        return 0;
}
