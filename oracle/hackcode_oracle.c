/*
 * hackcode_oracle.c -- CPU oracle for the hackcode1 Barnes-Hut hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, the
 * drop-in programs, the Python host mirror) may link, import or call this
 * file.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg use it, and only as the checker / the timed CPU reference arm.
 *
 * It is a plain-C FP64 restatement of the reference algorithm, written from
 * its published behaviour; each function names the reference file:line it
 * follows (paths inside the NEMO source tree).  Parity is pinned two ways
 * (see tests/test_oracle_golden.py):
 *   - against the reference's own golden vectors (hackcode1 Testfile bsf,
 *     nemo.bench h0 / p0 bsf, mkplummer Testfile bsf, bench12 nttot, the
 *     man-page log table), and
 *   - against oracle/_ref, the reference's load.c / grav.c / ran3.c compiled
 *     unchanged, tree-for-tree and force-for-force (bit-exact).
 *
 * Build: compiled with -ffp-contract=off so that no multiply-add is fused;
 * the reference's FP64 expressions are evaluated exactly as written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define NSUB 8
#define IMAX_ (1 << 30)          /* defs.h:124-128 (IMAX on 32-bit int) */

/* ------------------------------------------------------------------ */
/* RNG: NEMO's portable ran3 (Knuth subtractive generator, NumRec     */
/* ran3 variant) driven by xrandom.  src/kernel/numrec/ran3.c:43-94,  */
/* src/kernel/misc/xrandom.c:90-215 (NUMREC branch).                  */
/* ------------------------------------------------------------------ */

#define R3_MBIG 1000000000
#define R3_MSEED 161803398

static int r3_inext, r3_inextp, r3_ma[56], r3_first = 1;
static int r3_idum;

static double r3_next(int *idum)
{
    int mj, mk, i, ii, k;
    if (*idum < 0 || r3_first) {
        r3_first = 0;
        mj = R3_MSEED - (*idum < 0 ? -*idum : *idum);
        while (mj < 0) mj += R3_MBIG;
        mj %= R3_MBIG;
        r3_ma[55] = mj;
        mk = 1;
        for (i = 1; i <= 54; i++) {
            ii = (21 * i) % 55;
            r3_ma[ii] = mk;
            mk = mj - mk;
            while (mk < 0) mk += R3_MBIG;
            mj = r3_ma[ii];
        }
        for (k = 1; k <= 4; k++)
            for (i = 1; i <= 55; i++) {
                r3_ma[i] -= r3_ma[1 + (i + 30) % 55];
                if (r3_ma[i] < 0) r3_ma[i] += R3_MBIG;
            }
        r3_inext = 0;
        r3_inextp = 31;
        *idum = 1;
    }
    if (++r3_inext == 56) r3_inext = 1;
    if (++r3_inextp == 56) r3_inextp = 1;
    mj = r3_ma[r3_inext] - r3_ma[r3_inextp];
    while (mj < 0) mj += R3_MBIG;
    r3_ma[r3_inext] = mj;
    return mj * (1.0 / R3_MBIG);
}

/* set_xrandom(seed>0): xrandom.c:147-195 -- seeds ran3 with -seed once. */
void hco_xrandom_init(int seed)
{
    r3_idum = seed > 0 ? -seed : seed;
    r3_first = 1;
    r3_next(&r3_idum);
    r3_idum = 0;
}

/* xrandom(xl, xh): xrandom.c:197-215. */
double hco_xrandom(double xl, double xh)
{
    double r;
    if (xl == xh) return xl;
    r = r3_next(&r3_idum);
    return xl + r * (xh - xl);
}

/* ------------------------------------------------------------------ */
/* Initial conditions                                                 */
/* ------------------------------------------------------------------ */

/* pickball / pickshell: src/nbody/cores/pickpnt.c:14-48 */
static void pickshell(double *v, double rad)
{
    double rsq, rscale;
    int i;
    do {
        rsq = 0.0;
        for (i = 0; i < 3; i++) {
            v[i] = hco_xrandom(-1.0, 1.0);
            rsq = rsq + v[i] * v[i];
        }
    } while (rsq > 1.0);
    rscale = rad / sqrt(rsq);
    for (i = 0; i < 3; i++) v[i] = v[i] * rscale;
}

static void pickball(double *v, double rad)
{
    double rsq;
    int i;
    do {
        rsq = 0.0;
        for (i = 0; i < 3; i++) {
            v[i] = hco_xrandom(-1.0, 1.0);
            rsq = rsq + v[i] * v[i];
        }
    } while (rsq > 1.0);
    for (i = 0; i < 3; i++) v[i] = v[i] * rad;
}

/* pickvec: hackcode1/util.c:15-27 */
static void pickvec(double *x, int cf)
{
    if (cf) pickshell(x, hco_xrandom(0.0, 1.0));
    else pickball(x, 1.0);
}

/* make_testdata: hackcode1/code.c:129-153 (nbody= initial conditions).
 * phase is [n][2][3] (pos, vel). */
void hco_make_testdata(int n, int seed, int cencon, double *mass, double *phase)
{
    double cmr[3] = {0, 0, 0}, cmv[3] = {0, 0, 0};
    int i, k;
    hco_xrandom_init(seed);
    for (i = 0; i < n; i++) {
        double *x = phase + 6 * i, *v = x + 3;
        mass[i] = 1.0 / n;
        pickvec(x, cencon);
        for (k = 0; k < 3; k++) cmr[k] = cmr[k] + x[k];
        pickvec(v, 0);
        for (k = 0; k < 3; k++) cmv[k] = cmv[k] + v[k];
    }
    for (k = 0; k < 3; k++) { cmr[k] = cmr[k] / (double)n; cmv[k] = cmv[k] / (double)n; }
    for (i = 0; i < n; i++) {
        double *x = phase + 6 * i, *v = x + 3;
        for (k = 0; k < 3; k++) { x[k] = x[k] - cmr[k]; v[k] = v[k] - cmv[k]; }
    }
}

/* mkplummer with its defaults (mlow=0, mfrac=0.999, rfrac=22.8042468,
 * scale=-1 virial, quiet=0, zerocm=t, no mass spectrum):
 * src/nbody/init/mkplummer.c:49-71 (defaults), 257-422 (algorithm). */
void hco_mkplummer(int n, int seed, double *mass, double *phase)
{
    const double PI_ = 3.141592653589793238462643, TWO_PI_ = 6.283185307179586476925287;
    double mlow = 0.0, mfrac = 0.999, rfrac = 22.8042468;
    double scalefactor = 16.0 / (3.0 * PI_);
    double inv_scalefactor = 1.0 / scalefactor, sqrt_scalefactor = sqrt(scalefactor);
    double mrfrac, mtot = 0.0, radius, velocity, theta, phi, x, y;
    double w_sum, w_pos[3], w_vel[3];
    int i, k;

    hco_xrandom_init(seed);
    rfrac *= scalefactor;
    mrfrac = rfrac * rfrac * rfrac / pow(1.0 + rfrac * rfrac, 1.5);
    if (mrfrac < mfrac) mfrac = mrfrac;
    for (i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        mass[i] = 1.0 / (double)n;
        mtot += mass[i];
        radius = 1.0 / sqrt(pow(hco_xrandom(mlow, mfrac), -2.0 / 3.0) - 1.0);
        theta = acos(hco_xrandom(-1.0, 1.0));
        phi = hco_xrandom(0.0, TWO_PI_);
        p[0] = radius * sin(theta) * cos(phi);
        p[1] = radius * sin(theta) * sin(phi);
        p[2] = radius * cos(theta);
        x = 0.0;
        y = 0.1;
        while (y > x * x * pow(1.0 - x * x, 3.5)) {
            x = hco_xrandom(0.0, 1.0);
            y = hco_xrandom(0.0, 0.1);
        }
        velocity = x * sqrt(2.0) * pow(1.0 + radius * radius, -0.25);
        theta = acos(hco_xrandom(-1.0, 1.0));
        phi = hco_xrandom(0.0, TWO_PI_);
        v[0] = velocity * sin(theta) * cos(phi);
        v[1] = velocity * sin(theta) * sin(phi);
        v[2] = velocity * cos(theta);
    }
    for (i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        mass[i] /= mtot;
        for (k = 0; k < 3; k++) { p[k] = p[k] * inv_scalefactor; v[k] = v[k] * sqrt_scalefactor; }
    }
    w_sum = 0.0;
    for (k = 0; k < 3; k++) w_pos[k] = w_vel[k] = 0.0;
    for (i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        w_sum = w_sum + 1.0;
        for (k = 0; k < 3; k++) { w_pos[k] = w_pos[k] + p[k]; w_vel[k] = w_vel[k] + v[k]; }
    }
    for (k = 0; k < 3; k++) { w_pos[k] = w_pos[k] / w_sum; w_vel[k] = w_vel[k] / w_sum; }
    for (i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        for (k = 0; k < 3; k++) { p[k] = p[k] - w_pos[k]; v[k] = v[k] - w_vel[k]; }
    }
}

/* ------------------------------------------------------------------ */
/* Tree                                                               */
/* Node handles: 0 = empty, +k = body k-1, -k = cell k-1.             */
/* ------------------------------------------------------------------ */

typedef struct hco_tree {
    int nbody, maxcell, ncell, troot;
    int status;                 /* 0 ok, 1 cell overflow, 2 coincident */
    double rmin[3], rsize;
    const double *mass, *pos;   /* bodies (not owned) */
    int *sub;                   /* [maxcell][8] */
    double *cmass, *cpos, *cquad; /* [maxcell], [maxcell][3], [maxcell][9] */
    int *clevel;                /* depth of each cell (root = 0) */
} hco_tree;

hco_tree *hco_tree_new(int nbody, double fcells)
{
    hco_tree *t = (hco_tree *)calloc(1, sizeof(hco_tree));
    int mc = (int)(fcells * nbody);    /* load.c:50  maxcell = fcells * nbody */
    if (mc < 1) mc = 1;
    t->maxcell = mc;
    t->sub = (int *)malloc(sizeof(int) * 8 * (size_t)mc);
    t->cmass = (double *)malloc(sizeof(double) * (size_t)mc);
    t->cpos = (double *)malloc(sizeof(double) * 3 * (size_t)mc);
    t->cquad = (double *)malloc(sizeof(double) * 9 * (size_t)mc);
    t->clevel = (int *)malloc(sizeof(int) * (size_t)mc);
    t->rmin[0] = t->rmin[1] = t->rmin[2] = -2.0;
    t->rsize = 4.0;
    return t;
}

void hco_tree_free(hco_tree *t)
{
    if (!t) return;
    free(t->sub); free(t->cmass); free(t->cpos); free(t->cquad); free(t->clevel);
    free(t);
}

void hco_tree_set_box(hco_tree *t, const double *rmin, double rsize)
{
    t->rmin[0] = rmin[0]; t->rmin[1] = rmin[1]; t->rmin[2] = rmin[2];
    t->rsize = rsize;
}

void hco_tree_get_box(const hco_tree *t, double *rmin, double *rsize)
{
    rmin[0] = t->rmin[0]; rmin[1] = t->rmin[1]; rmin[2] = t->rmin[2];
    *rsize = t->rsize;
}

int hco_tree_ncell(const hco_tree *t) { return t->ncell; }
int hco_tree_status(const hco_tree *t) { return t->status; }

/* intcoord: load.c:135-156 */
static int intcoord(const hco_tree *t, int *xp, const double *rp)
{
    int k, inb = 1;
    double xsc;
    for (k = 0; k < 3; k++) {
        xsc = (rp[k] - t->rmin[k]) / t->rsize;
        if (0.0 <= xsc && xsc < 1.0) xp[k] = (int)floor(IMAX_ * xsc);
        else inb = 0;
    }
    return inb;
}

/* subindex: load.c:162-177 */
static int subindex(const int *x, int l)
{
    int i = 0, k;
    for (k = 0; k < 3; k++)
        if (x[k] & l) i += NSUB >> (k + 1);
    return i;
}

/* makecell: load.c:232-248 (bump allocator; overflow is an error) */
static int makecell(hco_tree *t)
{
    int c, i;
    if (t->ncell >= t->maxcell) { t->status = 1; return 0; }
    c = t->ncell++;
    for (i = 0; i < NSUB; i++) t->sub[8 * c + i] = 0;
    return -(c + 1);
}

/* expandbox: load.c:68-95 */
static void expandbox(hco_tree *t, int b)
{
    int k, xtmp[3], xmid[3];
    double rmid[3];
    const double *x = t->pos + 3 * b;
    while (!intcoord(t, xtmp, x)) {
        for (k = 0; k < 3; k++) rmid[k] = t->rmin[k] + 0.5 * t->rsize;
        for (k = 0; k < 3; k++)
            if (x[k] < rmid[k]) t->rmin[k] -= t->rsize;
        t->rsize = 2.0 * t->rsize;
        if (t->troot != 0) {
            int newt = makecell(t);
            if (t->status) return;
            intcoord(t, xmid, rmid);
            k = subindex(xmid, IMAX_ >> 1);
            t->sub[8 * (-newt - 1) + k] = t->troot;
            t->troot = newt;
        }
    }
}

/* loadtree: load.c:101-128 */
static void loadtree(hco_tree *t, int b)
{
    int l, xp[3], xq[3];
    int *qptr;
    intcoord(t, xp, t->pos + 3 * b);
    l = IMAX_ >> 1;
    qptr = &t->troot;
    while (*qptr != 0) {
        if (l == 0) { t->status = 2; return; }   /* assert(l != 0), load.c:113 */
        if (*qptr > 0) {
            int q = *qptr - 1, c = makecell(t);
            if (t->status) return;
            intcoord(t, xq, t->pos + 3 * q);
            t->sub[8 * (-c - 1) + subindex(xq, l)] = *qptr;
            *qptr = c;
        }
        qptr = &t->sub[8 * (-*qptr - 1) + subindex(xp, l)];
        l = l >> 1;
    }
    *qptr = b + 1;
}

/* hackcofm: load.c:183-226 (post-order; quadrupole under QUADPOLE). */
static void hackcofm(hco_tree *t, int q, int level, int usequad)
{
    int i, j, k, c;
    if (q >= 0) return;
    c = -q - 1;
    t->clevel[c] = level;
    double *cp = t->cpos + 3 * c, *Q = t->cquad + 9 * c;
    t->cmass[c] = 0.0;
    cp[0] = cp[1] = cp[2] = 0.0;
    for (i = 0; i < NSUB; i++) {
        int r = t->sub[8 * c + i];
        if (r != 0) {
            double m, tmpv[3];
            const double *rp;
            hackcofm(t, r, level + 1, usequad);
            if (r > 0) { m = t->mass[r - 1]; rp = t->pos + 3 * (r - 1); }
            else { m = t->cmass[-r - 1]; rp = t->cpos + 3 * (-r - 1); }
            t->cmass[c] += m;
            for (k = 0; k < 3; k++) tmpv[k] = rp[k] * m;
            for (k = 0; k < 3; k++) cp[k] = cp[k] + tmpv[k];
        }
    }
    for (k = 0; k < 3; k++) cp[k] = cp[k] / t->cmass[c];
    for (k = 0; k < 9; k++) Q[k] = 0.0;
    if (!usequad) return;
    for (i = 0; i < NSUB; i++) {
        int r = t->sub[8 * c + i];
        if (r != 0) {
            double m, dr[3], drsq, tmpm[9];
            const double *rp;
            if (r > 0) { m = t->mass[r - 1]; rp = t->pos + 3 * (r - 1); }
            else { m = t->cmass[-r - 1]; rp = t->cpos + 3 * (-r - 1); }
            for (k = 0; k < 3; k++) dr[k] = rp[k] - cp[k];
            drsq = dr[0] * dr[0];
            drsq += dr[1] * dr[1];
            drsq += dr[2] * dr[2];
            for (j = 0; j < 3; j++)
                for (k = 0; k < 3; k++) {
                    double drdr = dr[j] * dr[k];
                    double idrsq = (j == k ? 1.0 : 0.0) * drsq;
                    tmpm[3 * j + k] = drdr * 3.0;
                    tmpm[3 * j + k] = tmpm[3 * j + k] - idrsq;
                    tmpm[3 * j + k] = tmpm[3 * j + k] * m;
                }
            if (r < 0)
                for (k = 0; k < 9; k++) tmpm[k] = tmpm[k] + t->cquad[9 * (-r - 1) + k];
            for (k = 0; k < 9; k++) Q[k] = Q[k] + tmpm[k];
        }
    }
}

/* maketree: load.c:32-62.  Bodies with Mass == 0 are not loaded.
 * Returns 0, or 1 (cell overflow: "need more than maxcell cells"),
 * or 2 (two bodies share integer coordinates). */
int hco_maketree(hco_tree *t, int n, const double *mass, const double *pos, int usequad)
{
    int b;
    t->mass = mass;
    t->pos = pos;
    t->nbody = n;
    t->ncell = 0;
    t->troot = 0;
    t->status = 0;
    for (b = 0; b < n; b++)
        if (mass[b] != 0.0) {
            expandbox(t, b);
            if (t->status) return t->status;
            loadtree(t, b);
            if (t->status) return t->status;
        }
    if (t->troot < 0) hackcofm(t, t->troot, 0, usequad);
    return 0;
}

/* Tree dump for the structural parity check.  Per cell: its level, the
 * integer coordinates of its lower corner (30-bit grid of the root box),
 * the number of bodies below it, mass, centre of mass and the 6 unique
 * quadrupole components (xx, xy, xz, yy, yz, zz).  Per body: the level of
 * its parent cell (-1 for a lone root body or an unloaded body). */
static int count_dump(const hco_tree *t, int q, int level, int cx, int cy, int cz,
                      int *lev, int *corner, int *cnt, double *m, double *cm, double *quad,
                      int *bparent)
{
    int c = -q - 1, i, total = 0;
    int half = IMAX_ >> (level + 1);
    for (i = 0; i < NSUB; i++) {
        int r = t->sub[8 * c + i];
        int ox = cx + ((i & 4) ? half : 0), oy = cy + ((i & 2) ? half : 0), oz = cz + ((i & 1) ? half : 0);
        if (r > 0) { total += 1; if (bparent) bparent[r - 1] = level; }
        else if (r < 0)
            total += count_dump(t, r, level + 1, ox, oy, oz, lev, corner, cnt, m, cm, quad, bparent);
    }
    if (lev) lev[c] = level;
    if (corner) { corner[3 * c] = cx; corner[3 * c + 1] = cy; corner[3 * c + 2] = cz; }
    if (cnt) cnt[c] = total;
    if (m) m[c] = t->cmass[c];
    if (cm) { cm[3 * c] = t->cpos[3 * c]; cm[3 * c + 1] = t->cpos[3 * c + 1]; cm[3 * c + 2] = t->cpos[3 * c + 2]; }
    if (quad) {
        const double *Q = t->cquad + 9 * c;
        quad[6 * c + 0] = Q[0]; quad[6 * c + 1] = Q[1]; quad[6 * c + 2] = Q[2];
        quad[6 * c + 3] = Q[4]; quad[6 * c + 4] = Q[5]; quad[6 * c + 5] = Q[8];
    }
    return total;
}

int hco_tree_dump(const hco_tree *t, int *lev, int *corner, int *cnt, double *m, double *cm,
                  double *quad, int *bparent)
{
    int b;
    if (bparent) for (b = 0; b < t->nbody; b++) bparent[b] = -1;
    if (t->troot < 0)
        count_dump(t, t->troot, 0, 0, 0, 0, lev, corner, cnt, m, cm, quad, bparent);
    return t->ncell;
}

/* ------------------------------------------------------------------ */
/* Force walk: grav.c:22-131                                          */
/* ------------------------------------------------------------------ */

typedef struct {
    const hco_tree *t;
    double pos0[3], phi0, acc0[3], tolsq, eps2;
    int pskip;              /* node handle to skip (+b+1) or 0 */
    int usequad;
    int64_t n2b, nbc;
} walkstate;

/* gravsub: grav.c:42-73 */
static void gravsub(walkstate *w, int p, const double *dr_in, double drsq_in)
{
    const hco_tree *t = w->t;
    double dr[3], drsq, drabs, phii, mor3, m;
    int k;
    const double *pp;
    if (p > 0) { m = t->mass[p - 1]; pp = t->pos + 3 * (p - 1); }
    else { m = t->cmass[-p - 1]; pp = t->cpos + 3 * (-p - 1); }
    if (dr_in) {
        dr[0] = dr_in[0]; dr[1] = dr_in[1]; dr[2] = dr_in[2];
        drsq = drsq_in;
    } else {
        for (k = 0; k < 3; k++) dr[k] = pp[k] - w->pos0[k];
        drsq = dr[0] * dr[0];
        drsq += dr[1] * dr[1];
        drsq += dr[2] * dr[2];
    }
    drsq += w->eps2;
    drabs = sqrt(drsq);
    phii = m / drabs;
    w->phi0 -= phii;
    mor3 = phii / drsq;
    for (k = 0; k < 3; k++) w->acc0[k] = w->acc0[k] + dr[k] * mor3;
    if (w->usequad && p < 0) {
        const double *Q = t->cquad + 9 * (-p - 1);
        double dr5inv, quaddr[3], drquaddr, phiquad;
        dr5inv = 1.0 / (drsq * drsq * drabs);
        for (k = 0; k < 3; k++) {
            quaddr[k] = 0.0;
            quaddr[k] += Q[3 * k + 0] * dr[0];
            quaddr[k] += Q[3 * k + 1] * dr[1];
            quaddr[k] += Q[3 * k + 2] * dr[2];
        }
        drquaddr = dr[0] * quaddr[0];
        drquaddr += dr[1] * quaddr[1];
        drquaddr += dr[2] * quaddr[2];
        phiquad = -0.5 * dr5inv * drquaddr;
        w->phi0 = w->phi0 + phiquad;
        phiquad = 5.0 * phiquad / drsq;
        for (k = 0; k < 3; k++) w->acc0[k] = w->acc0[k] - dr[k] * phiquad;
        for (k = 0; k < 3; k++) quaddr[k] = quaddr[k] * dr5inv;
        for (k = 0; k < 3; k++) w->acc0[k] = w->acc0[k] - quaddr[k];
    }
}

/* walksub + subdivp: grav.c:93-131 */
static void walksub(walkstate *w, int p, double dsq)
{
    const hco_tree *t = w->t;
    if (p < 0) {
        int c = -p - 1, k;
        const double *cp = t->cpos + 3 * c;
        double dr[3], drsq;
        for (k = 0; k < 3; k++) dr[k] = cp[k] - w->pos0[k];
        drsq = dr[0] * dr[0];
        drsq += dr[1] * dr[1];
        drsq += dr[2] * dr[2];
        if (w->tolsq * drsq < dsq) {
            for (k = 0; k < NSUB; k++) {
                int s = t->sub[8 * c + k];
                if (s != 0) walksub(w, s, dsq / 4.0);
            }
        } else if (p != w->pskip) {
            gravsub(w, p, dr, drsq);
            w->nbc++;
        }
    } else if (p != w->pskip) {
        gravsub(w, p, NULL, 0.0);
        w->n2b++;
    }
}

/* hackgrav for a list of field points (hackgrav grav.c:22-32 /
 * hackforce.c:206-213).  skip[i] is the body index that field point i must
 * exclude (its own body, as hackcode1 does) or -1 (hackforce test=).
 * Per-point interaction counts go to n2b / nbc when non-NULL. */
void hco_forces(const hco_tree *t, int ntest, const double *tpos, const int *skip,
                double tol, double eps, int usequad, double *acc, double *phi,
                int64_t *n2b, int64_t *nbc)
{
    int i;
    walkstate w;
    memset(&w, 0, sizeof(w));
    w.t = t;
    w.tolsq = tol * tol;
    w.eps2 = eps * eps;
    w.usequad = usequad;
    for (i = 0; i < ntest; i++) {
        w.pos0[0] = tpos[3 * i]; w.pos0[1] = tpos[3 * i + 1]; w.pos0[2] = tpos[3 * i + 2];
        w.phi0 = 0.0;
        w.acc0[0] = w.acc0[1] = w.acc0[2] = 0.0;
        w.pskip = (skip && skip[i] >= 0) ? skip[i] + 1 : 0;
        w.n2b = w.nbc = 0;
        if (t->troot != 0) walksub(&w, t->troot, t->rsize * t->rsize);
        phi[i] = w.phi0;
        acc[3 * i] = w.acc0[0]; acc[3 * i + 1] = w.acc0[1]; acc[3 * i + 2] = w.acc0[2];
        if (n2b) n2b[i] = w.n2b;
        if (nbc) nbc[i] = w.nbc;
    }
}

/* Exact FP64 direct sum (the tol=0 limit of the walk, grav.c:122-131 with
 * every cell opened), skipping body skip[i].  Used for force-error
 * statistics; pairwise order is body index order. */
void hco_direct(int n, const double *mass, const double *pos, int ntest, const double *tpos,
                const int *skip, double eps, double *acc, double *phi)
{
    int i, j, k;
    double eps2 = eps * eps;
    for (i = 0; i < ntest; i++) {
        double a[3] = {0, 0, 0}, p = 0.0;
        for (j = 0; j < n; j++) {
            double dr[3], r2, r, phii, mor3;
            if ((skip && skip[i] == j) || mass[j] == 0.0) continue;
            for (k = 0; k < 3; k++) dr[k] = pos[3 * j + k] - tpos[3 * i + k];
            r2 = dr[0] * dr[0];
            r2 += dr[1] * dr[1];
            r2 += dr[2] * dr[2];
            r2 += eps2;
            r = sqrt(r2);
            phii = mass[j] / r;
            p -= phii;
            mor3 = phii / r2;
            for (k = 0; k < 3; k++) a[k] = a[k] + dr[k] * mor3;
        }
        phi[i] = p;
        acc[3 * i] = a[0]; acc[3 * i + 1] = a[1]; acc[3 * i + 2] = a[2];
    }
}

/* ------------------------------------------------------------------ */
/* hackcode1 run: startrun/stepsystem/output/diagnostics              */
/* code.c:57-64,159-191; code_io.c:111-197                            */
/* ------------------------------------------------------------------ */

/* Accumulator of every double the run writes to out= (bsf statistic:
 * src/kernel/io/bsf.c:114-160, moment.c:384-405). */
typedef struct {
    int64_t n;
    double sum1, sum2, vmin, vmax;
} hco_bsf;

static void bsf_add(hco_bsf *s, double v)
{
    if (s->n == 0) { s->vmin = v; s->vmax = v; }
    if (v < s->vmin) s->vmin = v;
    if (v > s->vmax) s->vmax = v;
    s->sum1 += v;
    s->sum2 += v * v;
    s->n++;
}

typedef struct {
    double freq, eps, tol, fcells, tstop, freqout, minor_freqout;
    int usequad;
    int opt_mass, opt_phi, opt_acc;   /* options= words (scanopt) */
    int write_out;                   /* 1: out= given */
} hco_params;

/* One log block per step (code_io.c:119-129). */
typedef struct {
    double tnow, etot[3], cmphase[6];
    int64_t nttot, n2b, nbc;
    int nbavg, ncavg;
} hco_logrow;

typedef struct {
    double etot[3], keten[9], peten[9], amten[9], cmphase[6], mtot;
} hco_diag;

/* diagnostics: code_io.c:160-197 */
static void diagnostics(int n, const double *mass, const double *pos, const double *vel,
                        const double *acc, const double *phi, hco_diag *d)
{
    int i, j, k;
    double velsq, tmpv[3], tmpt[9];
    memset(d, 0, sizeof(*d));
    for (i = 0; i < n; i++) {
        const double *x = pos + 3 * i, *v = vel + 3 * i, *a = acc + 3 * i;
        double m = mass[i];
        d->mtot += m;
        velsq = v[0] * v[0];
        velsq += v[1] * v[1];
        velsq += v[2] * v[2];
        d->etot[1] += 0.5 * m * velsq;
        d->etot[2] += 0.5 * m * phi[i];
        for (k = 0; k < 3; k++) tmpv[k] = v[k] * (0.5 * m);
        for (j = 0; j < 3; j++) for (k = 0; k < 3; k++) tmpt[3 * j + k] = tmpv[j] * v[k];
        for (k = 0; k < 9; k++) d->keten[k] = d->keten[k] + tmpt[k];
        for (k = 0; k < 3; k++) tmpv[k] = x[k] * m;
        for (j = 0; j < 3; j++) for (k = 0; k < 3; k++) tmpt[3 * j + k] = tmpv[j] * a[k];
        for (k = 0; k < 9; k++) d->peten[k] = d->peten[k] + tmpt[k];
        for (j = 0; j < 3; j++) for (k = 0; k < 3; k++) tmpt[3 * j + k] = tmpv[j] * v[k];
        for (k = 0; k < 9; k++) d->amten[k] = d->amten[k] + tmpt[k];
        for (k = 0; k < 3; k++) tmpv[k] = x[k] * m;
        for (k = 0; k < 3; k++) d->cmphase[k] = d->cmphase[k] + tmpv[k];
        for (k = 0; k < 3; k++) tmpv[k] = v[k] * m;
        for (k = 0; k < 3; k++) d->cmphase[3 + k] = d->cmphase[3 + k] + tmpv[k];
    }
    d->etot[0] = d->etot[1] + d->etot[2];
    for (j = 0; j < 3; j++) for (k = 0; k < 3; k++) tmpt[3 * j + k] = d->amten[3 * k + j];
    for (k = 0; k < 9; k++) d->amten[k] = d->amten[k] - tmpt[k];
    for (k = 0; k < 6; k++) d->cmphase[k] = d->cmphase[k] / d->mtot;
}

/* Optional record of every major output (PhaseSpace written): per output
 * 1 + 10 n doubles -- tnow, then phase [n][2][3], phi [n], acc [n][3] as
 * output() writes them (code_io.c:139-151).  Set before hco_hackcode1. */
static double *snap_sink = NULL;
static int snap_max = 0, snap_count = 0;

void hco_set_snapshot_sink(double *buf, int maxsnaps)
{
    snap_sink = buf;
    snap_max = buf ? maxsnaps : 0;
    snap_count = 0;
}

int hco_snapshot_count(void) { return snap_count; }

/* Run hackcode1 from given initial data.  phase [n][2][3] is updated in
 * place; acc [n][3] and phi [n] hold the last force evaluation.  Log rows
 * (at most maxrows) and the bsf statistic of out= are returned.  The
 * function returns the number of steps, or -1/-2 on tree errors. */
int hco_hackcode1(int n, const double *mass, double *phase, double *acc, double *phi,
                  double tnow, const hco_params *prm, hco_logrow *rows, int maxrows,
                  hco_bsf *bsf, double *box_rmin, double *box_rsize)
{
    double *pos = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *vel = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *tposbuf = pos;
    hco_tree *t = hco_tree_new(n, prm->fcells);
    double tout = tnow, minor_tout = tnow;
    int nstep = 0, i, k, firstmass = 1, nrow = 0;
    int64_t *n2b = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int64_t *nbc = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    int *skip = (int *)malloc(sizeof(int) * (size_t)n);
    double *anew = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    int rc = 0;

    for (i = 0; i < n; i++) {
        for (k = 0; k < 3; k++) { pos[3 * i + k] = phase[6 * i + k]; vel[3 * i + k] = phase[6 * i + 3 + k]; }
        skip[i] = i;
    }
    memset(acc, 0, sizeof(double) * 3 * (size_t)n);
    memset(phi, 0, sizeof(double) * (size_t)n);
    if (bsf) memset(bsf, 0, sizeof(*bsf));

    while (tnow < prm->tstop + 0.1 / prm->freq) {
        double dt = 1.0 / prm->freq, dthf = 0.5 * dt;
        int64_t n2bcalc = 0, nbccalc = 0, nfcalc = 0;
        hco_diag d;
        int bits = 0;
        if (hco_maketree(t, n, mass, pos, prm->usequad)) { rc = -t->status; break; }
        hco_forces(t, n, tposbuf, skip, prm->tol, prm->eps, prm->usequad, anew, phi, n2b, nbc);
        for (i = 0; i < n; i++) {
            nfcalc++;
            n2bcalc += n2b[i];
            nbccalc += nbc[i];
            if (nstep > 0)
                for (k = 0; k < 3; k++) {
                    double dacc = anew[3 * i + k] - acc[3 * i + k];
                    vel[3 * i + k] = vel[3 * i + k] + dacc * dthf;
                }
            for (k = 0; k < 3; k++) acc[3 * i + k] = anew[3 * i + k];
        }
        /* output(): code_io.c:111-154 */
        diagnostics(n, mass, pos, vel, acc, phi, &d);
        if (rows && nrow < maxrows) {
            hco_logrow *r = rows + nrow;
            r->tnow = tnow;
            memcpy(r->etot, d.etot, sizeof(d.etot));
            memcpy(r->cmphase, d.cmphase, sizeof(d.cmphase));
            r->n2b = n2bcalc;
            r->nbc = nbccalc;
            r->nttot = n2bcalc + nbccalc;
            r->nbavg = (int)((double)n2bcalc / (double)nfcalc);
            r->ncavg = (int)((double)nbccalc / (double)nfcalc);
        }
        nrow++;
        if (prm->minor_freqout > 0.0 && (minor_tout - 0.01 / prm->freq) <= tnow) {
            minor_tout += 1.0 / prm->minor_freqout;
            bits |= 1;                            /* TimeBit */
        }
        if (prm->freqout > 0.0 && (tout - 0.01 / prm->freq) <= tnow) {
            tout += 1.0 / prm->freqout;
            bits |= 1 | 2;                        /* TimeBit | PhaseSpaceBit */
            if (prm->opt_mass || firstmass) { bits |= 4; firstmass = 0; }
            if (prm->opt_phi) bits |= 8;
            if (prm->opt_acc) bits |= 16;
        }
        if (bits && prm->write_out && bsf) {
            /* put_snap order: Parameters(Time), Particles(Mass, PhaseSpace,
             * Potential, Acceleration), Diagnostics (code_io.c:203-216). */
            bsf_add(bsf, tnow);
            if (bits & 4) for (i = 0; i < n; i++) bsf_add(bsf, mass[i]);
            if (bits & 2)
                for (i = 0; i < n; i++) {
                    for (k = 0; k < 3; k++) bsf_add(bsf, pos[3 * i + k]);
                    for (k = 0; k < 3; k++) bsf_add(bsf, vel[3 * i + k]);
                }
            if (bits & 8) for (i = 0; i < n; i++) bsf_add(bsf, phi[i]);
            if (bits & 16) for (i = 0; i < 3 * n; i++) bsf_add(bsf, acc[i]);
            for (k = 0; k < 3; k++) bsf_add(bsf, d.etot[k]);
            for (k = 0; k < 9; k++) bsf_add(bsf, d.keten[k]);
            for (k = 0; k < 9; k++) bsf_add(bsf, d.peten[k]);
            for (k = 0; k < 9; k++) bsf_add(bsf, d.amten[k]);
            for (k = 0; k < 6; k++) bsf_add(bsf, d.cmphase[k]);
        }
        if ((bits & 2) && snap_sink && snap_count < snap_max) {
            double *o = snap_sink + (size_t)snap_count * (1 + 10 * (size_t)n);
            o[0] = tnow;
            for (i = 0; i < n; i++)
                for (k = 0; k < 3; k++) {
                    o[1 + 6 * i + k] = pos[3 * i + k];
                    o[1 + 6 * i + 3 + k] = vel[3 * i + k];
                }
            memcpy(o + 1 + 6 * (size_t)n, phi, sizeof(double) * (size_t)n);
            memcpy(o + 1 + 7 * (size_t)n, acc, sizeof(double) * 3 * (size_t)n);
            snap_count++;
        }
        /* kick-drift-kick remainder: code.c:182-188 */
        for (i = 0; i < n; i++)
            for (k = 0; k < 3; k++) {
                double dvel = acc[3 * i + k] * dthf;
                double vel1 = vel[3 * i + k] + dvel;
                double dpos = vel1 * dt;
                pos[3 * i + k] = pos[3 * i + k] + dpos;
                vel[3 * i + k] = vel1 + dvel;
            }
        nstep++;
        tnow = tnow + dt;
    }
    for (i = 0; i < n; i++)
        for (k = 0; k < 3; k++) { phase[6 * i + k] = pos[3 * i + k]; phase[6 * i + 3 + k] = vel[3 * i + k]; }
    if (box_rmin) hco_tree_get_box(t, box_rmin, box_rsize);
    hco_tree_free(t);
    free(pos); free(vel); free(n2b); free(nbc); free(skip); free(anew);
    return rc ? rc : nrow;
}

/* Diagnostics of a given state (code_io.c:160-197) for checks. */
void hco_diagnostics(int n, const double *mass, const double *phase, const double *acc,
                     const double *phi, double *out /* 3+9+9+9+6+1 */)
{
    double *pos = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double *vel = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    hco_diag d;
    int i, k;
    for (i = 0; i < n; i++)
        for (k = 0; k < 3; k++) { pos[3 * i + k] = phase[6 * i + k]; vel[3 * i + k] = phase[6 * i + 3 + k]; }
    diagnostics(n, mass, pos, vel, acc, phi, &d);
    memcpy(out, d.etot, 3 * sizeof(double));
    memcpy(out + 3, d.keten, 9 * sizeof(double));
    memcpy(out + 12, d.peten, 9 * sizeof(double));
    memcpy(out + 21, d.amten, 9 * sizeof(double));
    memcpy(out + 30, d.cmphase, 6 * sizeof(double));
    out[36] = d.mtot;
    free(pos); free(vel);
}

/* Layout sizes for ctypes mirrors. */
int hco_sizeof_logrow(void) { return (int)sizeof(hco_logrow); }
int hco_sizeof_params(void) { return (int)sizeof(hco_params); }
int hco_sizeof_bsf(void) { return (int)sizeof(hco_bsf); }
