// galaxy_model.h -- the composite disk galaxy: its constants, the tables its
// sampling reads, and the per-body sampling steps, shared by the host
// generator (galaxy.cpp, ran3 draws) and the device generator (hc_gen.cu,
// counter-based draws).  The model is described in galaxy.cpp.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define GAL_HD __host__ __device__ __forceinline__
#else
#define GAL_HD inline
#endif

namespace galaxy {

constexpr double PI = 3.141592653589793238462643;
constexpr double MD = 0.1, RD = 1.0, Z0 = 0.1, QT = 1.5, RDMAX = 15.0;
constexpr double MB = 0.033, AB = 0.2;
constexpr double MV = 1.0, RV = 30.0, CC = 10.0, RS = RV / CC;
constexpr int KG = 4000;     // potential grid, log-spaced in [1e-6, 1e4]
constexpr int NX = 8192;     // cumulative-mass inversion tables
constexpr int KR = 4096;     // disk kinematics, linear in [0, RDMAX R_d]
constexpr int JE = 1200;     // distribution function, log-spaced in E
constexpr int KB = 2048;     // rejection bounds, log-spaced radii in [1e-6, RV]
constexpr int TRIES = 1000000;

// the tables as plain pointers (host or device memory); component 0 is the
// bulge, 1 the halo
struct View {
    const double *r, *psi;                         // psi(r), decreasing
    double mtot, lr0, lr1;                         // total mass; log r[0], log r[KG-1]
    const double *xr, *xm;                         // disk: R / R_d against cumulative mass
    const double *tsr, *tsphi, *tsz, *tvphi;       // disk: sigma_R, sigma_phi, sigma_z, mean v_phi
    const double *dfE[2], *dff[2];                 // f(E), E decreasing
    const double *rr[2], *mm[2];                   // r against cumulative mass fraction
    const double *bnd[2];                          // max_v v^2 f(psi - v^2/2) per radius
    double mcomp[2];                               // component masses
};

GAL_HD double psi_at(const View &t, double x)
{
    if (x <= t.r[0]) return t.psi[0];
    if (x >= t.r[KG - 1]) return t.mtot / x;
    const double s = (log(x) - t.lr0) / (t.lr1 - t.lr0) * (double)(KG - 1);
    const int i = (int)s < KG - 2 ? (int)s : KG - 2;
    const double w = s - (double)i;
    return t.psi[i] * (1.0 - w) + t.psi[i + 1] * w;
}

GAL_HD double df_at(const double *E, const double *f, double e)
{
    if (e <= E[JE - 1]) return 0.0;
    if (e >= E[0]) return f[0];
    int lo = 0, hi = JE - 1;                       // E decreasing: bisection
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (E[mid] > e) lo = mid;
        else hi = mid;
    }
    const double w = (e - E[hi]) / (E[lo] - E[hi]);
    return f[hi] + w * (f[lo] - f[hi]);
}

// x at cumulative value u on a monotone table (linear interpolation; the
// first entry above u found by bisection)
GAL_HD double invert(const double *xx, const double *mm, int n, double u)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (mm[mid] > u) hi = mid;
        else lo = mid + 1;
    }
    if (lo == 0) return xx[0];
    if (lo >= n) return xx[n - 1];
    const double w = (u - mm[lo - 1]) / (mm[lo] - mm[lo - 1]);
    return xx[lo - 1] + w * (xx[lo] - xx[lo - 1]);
}

GAL_HD double disk_lerp(const double *tab, double R)
{
    const double x = R / (RD * RDMAX) * (KR - 1.0);
    const int k = (int)x < KR - 2 ? (int)x : KR - 2;
    const double w = x - k;
    return tab[k] * (1.0 - w) + tab[k + 1] * w;
}

// U: a uniform draw u(lo, hi) = lo + (hi - lo) * next
template <class U> GAL_HD double gauss(U &u)
{
    const double u1 = u(1e-300, 1.0), u2 = u(0.0, 2.0 * PI);      // Box-Muller
    return sqrt(-2.0 * log(u1)) * cos(u2);
}

template <class U> GAL_HD void iso_direction(U &u, double len, double *v)
{
    const double ct = u(-1.0, 1.0), st = sqrt(fmax(0.0, 1.0 - ct * ct));
    const double ph = u(0.0, 2.0 * PI);
    v[0] = len * st * cos(ph);
    v[1] = len * st * sin(ph);
    v[2] = len * ct;
}

// speed from g(v) = v^2 f(psi - v^2/2) by rejection under bound; 0 (and
// *fail set) after TRIES draws
template <class U> GAL_HD double sample_speed(U &u, const double *E, const double *f, double psi, double bound,
                                              bool *fail)
{
    const double vmax = sqrt(2.0 * psi);
    if (!(bound > 0.0)) return 0.0;
    for (int tries = 0; tries < TRIES; tries++) {
        const double v = u(0.0, vmax);
        if (u(0.0, bound) <= v * v * df_at(E, f, psi - 0.5 * v * v)) return v;
    }
    *fail = true;
    return 0.0;
}

// one disk body: R from the exponential profile, z from sech^2, Gaussian
// velocities about the asymmetric-drift-corrected rotation
template <class U> GAL_HD void disk_body(const View &t, U &u, double *p, double *v)
{
    const double R = RD * invert(t.xr, t.xm, NX, u(0.0, 1.0));
    const double ph = u(0.0, 2.0 * PI);
    double q = u(-1.0, 1.0);
    q = fmax(-1.0 + 1e-12, fmin(1.0 - 1e-12, q));
    p[0] = R * cos(ph);
    p[1] = R * sin(ph);
    p[2] = Z0 * atanh(q);
    const double sr = disk_lerp(t.tsr, R), sphi = disk_lerp(t.tsphi, R), sz = disk_lerp(t.tsz, R);
    const double vphi = disk_lerp(t.tvphi, R) + sphi * gauss(u);
    const double vr = sr * gauss(u), vz = sz * gauss(u);
    v[0] = vr * cos(ph) - vphi * sin(ph);
    v[1] = vr * sin(ph) + vphi * cos(ph);
    v[2] = vz;
}

// one bulge (c = 0) or halo (c = 1) body: radius from the cumulative mass,
// isotropic speed from the component's distribution function
template <class U> GAL_HD void sphere_body(const View &t, int c, U &u, double *p, double *v, bool *fail)
{
    const double rad = invert(t.rr[c], t.mm[c], NX, u(0.0, 1.0));
    iso_direction(u, rad, p);
    const double lb0 = log(1e-6), lb1 = log(RV);
    const double x = (log(fmax(rad, 1e-6)) - lb0) / (lb1 - lb0) * (KB - 1.0);
    int k = (int)x < KB - 2 ? (int)x : KB - 2;
    k = k > 0 ? k : 0;
    const double psi = psi_at(t, rad);
    const double b = 1.25 * fmax(t.bnd[c][k], t.bnd[c][k + 1]);
    iso_direction(u, sample_speed(u, t.dfE[c], t.dff[c], psi, b, fail), v);
}

// host-built tables (galaxy.cpp)
struct Tables {
    std::vector<double> r, psi, xr, xm, tsr, tsphi, tsz, tvphi;
    std::vector<double> dfE[2], dff[2], rr[2], mm[2], bnd[2];
    double mtot = 0.0, mcomp[2] = {MB, MV};
    View view() const;
};
void build_tables(Tables &t);

}  // namespace galaxy
