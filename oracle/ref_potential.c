/*
 * ref_potential.c -- driver around one of NEMO's potential plug-ins.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile links this file with one of the
 * reference's src/orbit/potential/data/{plummer,hernquist,miyamoto,log}.c,
 * compiled unchanged, into oracle/_ref/libpot_<name>.so: the plug-ins that
 * hackcode3's potname= loads (hackcode3/grav.c:34-38).  ref_pot_eval
 * initialises the plug-in with potpars (inipotential) and evaluates
 * potential_double at each point, for comparison with the GPU's field.
 */
#include <stdinc.h>
#include <stdarg.h>

/* libnemo services the plug-ins call */
int debug_level = 0;
static int quiet_dprintf(int lev, const_string fmt, ...) { (void)lev; (void)fmt; return 0; }
dprintf_pter get_dprintf(const_string f, int l) { (void)f; (void)l; return quiet_dprintf; }
void warning(string fmt, ...) { (void)fmt; }
void nemo_error(string fmt, ...) { (void)fmt; abort(); }

extern void inipotential(int *npar, double *par, string name);
extern void potential_double(int *ndim, double *pos, double *acc, double *pot, double *time);

/* par[0..npar) as potpars= gives them (pattern speed first); pos[3n] ->
 * acc[3n], pot[n] at time 0 */
int ref_pot_eval(int npar, const double *par, int n, const double *pos, double *acc, double *pot)
{
    int i, ndim = 3;
    double p[16], t = 0.0;
    if (npar > 16) return -1;
    for (i = 0; i < npar; i++) p[i] = par[i];
    inipotential(&npar, p, "ref");
    for (i = 0; i < n; i++) potential_double(&ndim, (double *)pos + 3 * i, acc + 3 * i, pot + i, &t);
    return n;
}
