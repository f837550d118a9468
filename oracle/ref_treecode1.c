/*
 * ref_treecode1.c -- driver around treecode1's setrcrit, for checks.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file, which
 * #includes the reference's src/nbody/evolve/hackcode/treecode1/treeload.c
 * unchanged (so that its file-local setrcrit, treeload.c:232-252, and the
 * bh86/sw94 flags it reads are in this translation unit), into
 * oracle/_ref/libtc1ref.so.  ref_setrcrit gives the reference's critical
 * radius^2 of cells described by their geometric centre, size and centre of
 * mass, for comparison with the GPU's per-cell radii of the same cells.
 */
#include <stdinc.h>
#include <mathfns.h>
#include <vectmath.h>
#define global /* define the treecode.h globals here, as treecode.c does */
#include "treecode.h"
#include "treeload.c"

/* libnemo services that treeload.c links against; setrcrit calls none of them */
int debug_level = 0;
void nemo_error(string fmt, ...) { (void)fmt; abort(); }
void *allocate_FL(size_t n, const_string file, int line) { (void)file; (void)line; return calloc(1, n ? n : 1); }
double cputime(void) { return 0.0; }
bool scanopt(string opt, string key) { (void)opt; (void)key; return FALSE; }

/* criterion: 1 bh86, 2 sw94, 3 the default ("new") criterion.  For cell i,
 * center[3i..3i+2] is its geometric centre, size[i] its side, cm[3i..] its
 * centre of mass; rcrit2[i] receives Rcrit2 as setrcrit assigns it. */
int ref_setrcrit(int criterion, double theta_, double rsize_, int ncell, const double *center,
                 const double *size, const double *cm, double *rcrit2)
{
    int i, k;
    cell c;
    vector cmpos;
    theta = theta_;
    rsize = rsize_;
    bh86 = criterion == 1;
    sw94 = criterion == 2;
    for (i = 0; i < ncell; i++) {
        memset(&c, 0, sizeof(c));
        for (k = 0; k < NDIM; k++) {
            Pos(&c)[k] = center[3 * i + k];
            cmpos[k] = cm[3 * i + k];
        }
        setrcrit(&c, cmpos, size[i]);
        rcrit2[i] = Rcrit2(&c);
    }
    return ncell;
}
