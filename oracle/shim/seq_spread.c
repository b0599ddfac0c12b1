/*
 * Test infrastructure only.  The reference's coloured spread
 * (old-version/spme_kernel.c:250-290) skips the last nb^3 mod 8 blocks when
 * nb = ceil(K/p) is odd and races across colours for some K, p.  The
 * reference ships a sequential variant of the same loop, commented out at
 * old-version/spme_kernel.c:292-297.  This file supplies `spread` with that
 * sequential loop (plus the mesh zeroing of :271-275) and calls the
 * reference's own spread_kernel; the coloured `spread` in spme_kernel.c is
 * renamed at compile time (-Dspread=...) so it stays unused.
 */
#include <string.h>

void spread_kernel(int porder3, double *P, int *ind, double *grid, int ld3,
                   double *forces);

void spread(int np, int nb, int *head, int *next, int porder3, double *P, int ldP,
            int *ind, int ldind, double *forces, double *grid, int ld3)
{
    int i;
    (void)nb; (void)head; (void)next;
    memset(grid, 0, sizeof(double) * (size_t)ld3 * 3);
    for (i = 0; i < np; i++)
        spread_kernel(porder3, &P[(long)i * ldP], &ind[(long)i * ldind], grid, ld3,
                      &forces[i * 3]);
}
