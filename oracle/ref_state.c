/*
 * ref_state.c -- driver around hackcode1's savestate / restorestate.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file, which
 * #includes the reference's hackcode1/code_io.c unchanged (savestate and
 * restorestate, code_io.c:222-284), and links it with NEMO's own filestruct
 * library sources (src/kernel/io/filesecret.c and the kernel files it calls:
 * extstring.c, convert.c, ieeehalfprecision.c, stropen.c,
 * src/kernel/cores/strlib.c, bswap.c) into oracle/_ref/libstateref.so.  It
 * lets tests write a state file exactly as the reference does and read one
 * with the reference's own reader.
 */
#define global /* define the code.h globals here, as code.c does */
#include "code_io.c"
#include <setjmp.h>
#include <stdarg.h>
#include <string.h>

string headline = "";

/* ---- libnemo services used here (getparam, errors, allocation, output) ---- */
int debug_level = 0;
static char argv0_buf[256] = "hackcode1", version_buf[64] = "1.5b";
static jmp_buf err_jmp;
static int err_armed = 0;
static char err_msg[512];

static int quiet_dprintf(int lev, const_string fmt, ...) { (void)lev; (void)fmt; return 0; }
dprintf_pter get_dprintf(const_string f, int l) { (void)f; (void)l; return quiet_dprintf; }
void nemo_error(string fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err_msg, sizeof(err_msg), fmt, ap);
    va_end(ap);
    if (err_armed) longjmp(err_jmp, 1);
    fprintf(stderr, "ref_state: fatal: %s\n", err_msg);
    abort();
}
void nemo_warning(string fmt, ...) { (void)fmt; }
void *allocate_FL(size_t n, const_string file, int line) { (void)file; (void)line; return calloc(1, n ? n : 1); }
void *reallocate_FL(void *p, size_t n, const_string file, int line) { (void)file; (void)line; return realloc(p, n); }
string getparam(string name)
{
    if (streq(name, "argv0")) return argv0_buf;
    if (streq(name, "VERSION")) return version_buf;
    return "";
}
/* not reached from savestate / restorestate */
double cputime(void) { return 0.0; }
bool scanopt(string opt, string key) { (void)opt; (void)key; return FALSE; }
int put_history(stream s) { (void)s; return 0; }
int get_history(stream s) { (void)s; return 0; }
string ask_headline(void) { return ""; }

const char *ref_state_error(void) { return err_msg; }

/* the program name (argv0) and VERSION keyword the state file records */
void ref_state_identity(const char *prog, const char *version)
{
    snprintf(argv0_buf, sizeof(argv0_buf), "%s", prog);
    snprintf(version_buf, sizeof(version_buf), "%s", version);
}

/* Write a state file with the reference's savestate.  dbl[12] = freq, tol,
 * eps, fcells, tstop, freqout, minor_freqout, tnow, tout, minor_tout, rsize,
 * (unused); rmin[3]; phase [n][2][3]. */
int ref_state_write(const char *file, const char *headline_, const char *options_, const double *dbl,
                    int nstep_, const double *rmin_, int n, const double *mass, const double *phase,
                    const double *acc, const double *phi)
{
    int i, k;
    headline = (string)headline_;
    options = (string)options_;
    freq = dbl[0]; tol = dbl[1]; eps = dbl[2]; fcells = dbl[3]; tstop = dbl[4]; freqout = dbl[5];
    minor_freqout = dbl[6]; tnow = dbl[7]; tout = dbl[8]; minor_tout = dbl[9]; rsize = dbl[10];
    nstep = nstep_;
    for (k = 0; k < NDIM; k++) rmin[k] = rmin_[k];
    nbody = n;
    bodytab = (bodyptr)calloc((size_t)n, sizeof(body));
    for (i = 0; i < n; i++) {
        bodyptr p = bodytab + i;
        Type(p) = BODY;
        Mass(p) = mass[i];
        for (k = 0; k < NDIM; k++) {
            Pos(p)[k] = phase[6 * i + k];
            Vel(p)[k] = phase[6 * i + 3 + k];
            Acc(p)[k] = acc[3 * i + k];
        }
        Phi(p) = phi[i];
    }
    err_armed = 1;
    if (setjmp(err_jmp)) { err_armed = 0; free(bodytab); return 1; }
    savestate((string)file);
    err_armed = 0;
    free(bodytab);
    bodytab = NULL;
    return 0;
}

/* Read a state file with the reference's restorestate: same layout as
 * ref_state_write; headline / options copied into buffers of `slen` bytes;
 * arrays sized for *n bodies on entry (the count read is returned in *n). */
int ref_state_read(const char *file, char *headline_, char *options_, int slen, double *dbl, int *nstep_,
                   double *rmin_, int *n, double *mass, double *phase, double *acc, double *phi)
{
    int i, k, cap = *n;
    err_armed = 1;
    if (setjmp(err_jmp)) { err_armed = 0; return 1; }
    logstr = stderr;
    restorestate((string)file);
    err_armed = 0;
    snprintf(headline_, slen, "%s", headline);
    snprintf(options_, slen, "%s", options);
    dbl[0] = freq; dbl[1] = tol; dbl[2] = eps; dbl[3] = fcells; dbl[4] = tstop; dbl[5] = freqout;
    dbl[6] = minor_freqout; dbl[7] = tnow; dbl[8] = tout; dbl[9] = minor_tout; dbl[10] = rsize;
    *nstep_ = nstep;
    for (k = 0; k < NDIM; k++) rmin_[k] = rmin[k];
    *n = nbody;
    if (nbody > cap) return 2;
    for (i = 0; i < nbody; i++) {
        bodyptr p = bodytab + i;
        mass[i] = Mass(p);
        for (k = 0; k < NDIM; k++) {
            phase[6 * i + k] = Pos(p)[k];
            phase[6 * i + 3 + k] = Vel(p)[k];
            acc[3 * i + k] = Acc(p)[k];
        }
        phi[i] = Phi(p);
    }
    return Type(bodytab) == BODY ? 0 : 3;
}
