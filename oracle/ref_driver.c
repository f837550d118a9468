/*
 * ref_driver.c -- thin driver around the reference's own tree and walk.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles the reference's
 * src/nbody/evolve/hackcode/hackcode1/load.c and grav.c and
 * src/kernel/numrec/ran3.c unchanged, from where they lie in the NEMO source
 * tree, and links them with this file into oracle/_ref/libhcref_{mp,qp}.so
 * (monopole / -DQUADPOLE builds, as hackcode1/Makefile:82-115 does).  This
 * driver supplies the globals that hackcode1/code.c would define and the few
 * libnemo services load.c/grav.c call (allocate, error, dprintf), then exposes
 * plain-C entry points so that tests can compare the oracle restatement with
 * the reference tree-for-tree and force-for-force.
 */
#define global /* define the code.h globals here, as code.c does */
#include "code.h"
#include <setjmp.h>
#include <stdarg.h>
#include <stdint.h>
#include <string.h>

/* code.c declares this; the walk never reads it. */
string headline = "ref_driver";

/* ---- libnemo services used by load.c / grav.c ---- */
int debug_level = 0;

static int quiet_dprintf(int lev, const_string fmt, ...) { (void)lev; (void)fmt; return 0; }
dprintf_pter get_dprintf(const_string f, int l) { (void)f; (void)l; return quiet_dprintf; }

static jmp_buf err_jmp;
static int err_armed = 0;
static char err_msg[256];

void nemo_error(string fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err_msg, sizeof(err_msg), fmt, ap);
    va_end(ap);
    if (err_armed) longjmp(err_jmp, 1);
    fprintf(stderr, "ref_driver: fatal: %s\n", err_msg);
    abort();
}

void *allocate_FL(size_t n, const_string file, int line)
{
    void *p;
    (void)file; (void)line;
    p = calloc(1, n ? n : 1);
    if (!p) nemo_error("allocate: out of memory");
    return p;
}

/* ---- state ---- */
static body *btab = NULL;
static int btab_n = 0;

const char *ref_error_message(void) { return err_msg; }
int ref_quadpole(void)
{
#ifdef QUADPOLE
    return 1;
#else
    return 0;
#endif
}

/* The reference allocates its cell pool once, on the first maketree call,
 * as fcells * nbody cells (load.c:49-53) and never frees it.  ref_init makes
 * that first call with max_nbody massless bodies so that later calls with up
 * to max_nbody bodies share one pool. */
int ref_init(int max_nbody, double fcells_)
{
    fcells = fcells_;
    btab = (body *)calloc((size_t)max_nbody, sizeof(body));
    btab_n = max_nbody;
    SETVS(rmin, -2.0);
    rsize = 4.0;
    /* two massive bodies (hackcofm needs a root), the rest massless */
    Mass(&btab[0]) = Mass(&btab[1]) = 1.0;
    Pos(&btab[1])[0] = 0.5;
    maketree(btab, max_nbody);
    Mass(&btab[0]) = Mass(&btab[1]) = 0.0;
    return 0;
}

/* Load bodies and build the tree (maketree, load.c:32-62) in the given
 * root box; the (possibly expanded) box is returned in place.  Returns 0 or
 * 1 when the reference called error() (cell pool exhausted). */
int ref_maketree(int n, const double *mass, const double *pos, double *box_rmin, double *box_rsize)
{
    int i, k, nmassive = 0;
    if (n > btab_n) return 2;
    for (i = 0; i < n; i++) nmassive += (mass[i] != 0.0);
    if (nmassive == 0) return 3;    /* load.c:61 would dereference a NULL root */
    for (i = 0; i < n; i++) {
        Type(&btab[i]) = BODY;
        Mass(&btab[i]) = mass[i];
        for (k = 0; k < NDIM; k++) Pos(&btab[i])[k] = pos[3 * i + k];
    }
    for (k = 0; k < NDIM; k++) rmin[k] = box_rmin[k];
    rsize = *box_rsize;
    err_armed = 1;
    if (setjmp(err_jmp)) { err_armed = 0; return 1; }
    maketree(btab, n);
    err_armed = 0;
    for (k = 0; k < NDIM; k++) box_rmin[k] = rmin[k];
    *box_rsize = rsize;
    return 0;
}

/* Tree dump in the same layout as hco_tree_dump (oracle), cells in DFS
 * pre-order with children in subindex order 0..7. */
static int dump_rec(nodeptr q, int level, int cx, int cy, int cz, int *ncell,
                    int *lev, int *corner, int *cnt, double *m, double *cm, double *quad,
                    int *bparent)
{
    int c = (*ncell)++, i, total = 0;
    int half = (IMAX) >> (level + 1);
    for (i = 0; i < NSUB; i++) {
        nodeptr r = Subp(q)[i];
        int ox = cx + ((i & 4) ? half : 0), oy = cy + ((i & 2) ? half : 0), oz = cz + ((i & 1) ? half : 0);
        if (r == NULL) continue;
        if (Type(r) == BODY) {
            total += 1;
            if (bparent) bparent[(bodyptr)r - btab] = level;
        } else
            total += dump_rec(r, level + 1, ox, oy, oz, ncell, lev, corner, cnt, m, cm, quad, bparent);
    }
    if (lev) lev[c] = level;
    if (corner) { corner[3 * c] = cx; corner[3 * c + 1] = cy; corner[3 * c + 2] = cz; }
    if (cnt) cnt[c] = total;
    if (m) m[c] = Mass(q);
    if (cm) for (i = 0; i < 3; i++) cm[3 * c + i] = Pos(q)[i];
#ifdef QUADPOLE
    if (quad) {
        quad[6 * c + 0] = Quad(q)[0][0]; quad[6 * c + 1] = Quad(q)[0][1];
        quad[6 * c + 2] = Quad(q)[0][2]; quad[6 * c + 3] = Quad(q)[1][1];
        quad[6 * c + 4] = Quad(q)[1][2]; quad[6 * c + 5] = Quad(q)[2][2];
    }
#else
    if (quad) for (i = 0; i < 6; i++) quad[6 * c + i] = 0.0;
#endif
    return total;
}

int ref_tree_dump(int n, int *lev, int *corner, int *cnt, double *m, double *cm, double *quad,
                  int *bparent)
{
    int ncell = 0, b;
    if (bparent) for (b = 0; b < n; b++) bparent[b] = -1;
    if (troot != NULL && Type(troot) == CELL)
        dump_rec(troot, 0, 0, 0, 0, &ncell, lev, corner, cnt, m, cm, quad, bparent);
    return ncell;
}

int ref_tree_ncell(void)
{
    int ncell = 0;
    if (troot != NULL && Type(troot) == CELL)
        dump_rec(troot, 0, 0, 0, 0, &ncell, NULL, NULL, NULL, NULL, NULL, NULL, NULL);
    return ncell;
}

/* hackgrav (grav.c:22-32) at body i of the loaded set (self skipped), or,
 * when ntest > 0 and tpos != NULL, at separate test points that are not in
 * the tree (hackforce test=, hackforce.c:206-213).  Per-point counts go to
 * n2b / nbc. */
int ref_forces(int n, int ntest, const double *tpos, double tol_, double eps_,
               double *acc, double *phi, int64_t *n2b, int64_t *nbc)
{
    int i, k;
    body tb;
    tol = tol_;
    eps = eps_;
    if (tpos == NULL) {
        for (i = 0; i < n; i++) {
            hackgrav(&btab[i]);
            phi[i] = Phi(&btab[i]);
            for (k = 0; k < NDIM; k++) acc[3 * i + k] = Acc(&btab[i])[k];
            if (n2b) n2b[i] = n2bterm;
            if (nbc) nbc[i] = nbcterm;
        }
        return n;
    }
    memset(&tb, 0, sizeof(tb));
    Type(&tb) = BODY;
    for (i = 0; i < ntest; i++) {
        for (k = 0; k < NDIM; k++) Pos(&tb)[k] = tpos[3 * i + k];
        hackgrav(&tb);
        phi[i] = Phi(&tb);
        for (k = 0; k < NDIM; k++) acc[3 * i + k] = Acc(&tb)[k];
        if (n2b) n2b[i] = n2bterm;
        if (nbc) nbc[i] = nbcterm;
    }
    return ntest;
}

/* hackgrav (grav.c:22-32) at the loaded bodies idx[0..nidx) only, each
 * skipping itself as hackcode1's force loop does (code.c:170-174): a sample
 * of a large system, or one worker's share of it. */
int ref_forces_idx(int nidx, const int *idx, double tol_, double eps_,
                   double *acc, double *phi, int64_t *n2b, int64_t *nbc)
{
    int i, k;
    tol = tol_;
    eps = eps_;
    for (i = 0; i < nidx; i++) {
        bodyptr p = &btab[idx[i]];
        hackgrav(p);
        phi[i] = Phi(p);
        for (k = 0; k < NDIM; k++) acc[3 * i + k] = Acc(p)[k];
        if (n2b) n2b[i] = n2bterm;
        if (nbc) nbc[i] = nbcterm;
    }
    return nidx;
}

/* ran3 as linked from the reference (ran3.c:43-94): fill out[] with the
 * first count deviates after seeding with -seed, as set_xrandom does. */
extern real ran3(int *);
void ref_ran3_sequence(int seed, int count, double *out)
{
    int idum = seed > 0 ? -seed : seed, i;
    ran3(&idum);          /* seeding call, value discarded (xrandom.c:183-186) */
    idum = 0;
    for (i = 0; i < count; i++) out[i] = ran3(&idum);
}
