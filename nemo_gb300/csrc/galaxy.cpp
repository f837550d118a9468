// galaxy.cpp -- composite disk galaxy initial conditions (project-written; no
// NEMO program draws this model the same way, so its parity is pinned only
// by the model's own moments).
//
// Model, G = 1:
//   disk   M_d = 0.1, exponential surface density Sigma0 exp(-R/R_d), R_d = 1,
//          vertical sech^2(z / z0), z0 = 0.1, truncated at R = 15 R_d;
//   bulge  Hernquist, M_b = 0.033 inside its truncation radius r_vir, a_b = 0.2;
//   halo   NFW, M_vir = 1 inside r_vir = 30, concentration c = 10 (r_s = 3),
//          truncated at r_vir.
// Potential: bulge and halo exactly (spherical); the disk's mass enclosed in
// a sphere, M_d (1 - (1 + r/R_d) e^{-r/R_d}), for the spherical potential the
// bulge and halo feel; the disk's own midplane rotation uses the exact
// exponential-disk curve v^2 = 4 pi Sigma0 R_d y^2 [I0 K0 - I1 K1](y),
// y = R / (2 R_d) (Freeman 1970).
// Velocities:
//   bulge, halo: isotropic, from the distribution function obtained by
//     Eddington's inversion f(E) = (1/(sqrt 8 pi^2)) d/dE int_0^E
//     (drho/dpsi) dpsi / sqrt(E - psi) in the total spherical potential
//     (tabulated on a logarithmic radius grid; f clamped at 0 where the
//     truncation makes it negative); speeds drawn by rejection;
//   disk: Gaussian in (v_R, v_phi, v_z) with sigma_R from Toomre's
//     Q = sigma_R kappa / (3.36 Sigma) = 1.5, sigma_phi^2 = sigma_R^2
//     kappa^2 / (4 Omega^2) (epicyclic), sigma_z^2 = pi Sigma z0 (isothermal
//     sheet), mean v_phi^2 = v_c^2 + sigma_R^2 (1 - kappa^2/(4 Omega^2) -
//     2 R / R_d) (asymmetric drift), rotating in the positive sense about z.
// Bodies: disk, then bulge, then halo; equal masses within each component;
// the centre of mass and its velocity are removed at the end.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#include "nemo_io.h"

namespace nemo {

namespace {

constexpr double PI = 3.141592653589793238462643;
constexpr double MD = 0.1, RD = 1.0, Z0 = 0.1, QT = 1.5, RDMAX = 15.0;
constexpr double MB = 0.033, AB = 0.2;
constexpr double MV = 1.0, RV = 30.0, CC = 10.0, RS = RV / CC;

double nfw_m(double x) { return std::log1p(x) - x / (1.0 + x); }

double m_bulge(double r)
{
    const double rr = std::min(r, RV);
    const double f = (rr * rr) / ((rr + AB) * (rr + AB)), ft = (RV * RV) / ((RV + AB) * (RV + AB));
    return MB * f / ft;
}
double rho_bulge(double r)
{
    if (r > RV) return 0.0;
    const double ft = (RV * RV) / ((RV + AB) * (RV + AB));
    return (MB / ft) * AB / (2.0 * PI * r * std::pow(r + AB, 3));
}
double m_halo(double r) { return MV * nfw_m(std::min(r, RV) / RS) / nfw_m(CC); }
double rho_halo(double r)
{
    if (r > RV) return 0.0;
    const double x = r / RS, rhos = MV / (4.0 * PI * RS * RS * RS * nfw_m(CC));
    return rhos / (x * (1.0 + x) * (1.0 + x));
}
double m_disk_sph(double r)
{
    const double x = std::min(r, RDMAX * RD) / RD;
    return MD * (1.0 - (1.0 + x) * std::exp(-x)) / (1.0 - (1.0 + RDMAX) * std::exp(-RDMAX));
}

struct Grid {
    std::vector<double> r, psi;          // psi decreasing with r
    double mtot = 0.0;
    double psi_at(double x) const
    {
        if (x <= r.front()) return psi.front();
        if (x >= r.back()) return mtot / x;
        const double lx = std::log(x), l0 = std::log(r.front()), l1 = std::log(r.back());
        const double t = (lx - l0) / (l1 - l0) * (double)(r.size() - 1);
        const size_t i = std::min((size_t)t, r.size() - 2);
        const double w = t - (double)i;
        return psi[i] * (1.0 - w) + psi[i + 1] * w;
    }
};

Grid make_grid()
{
    Grid g;
    const int K = 4000;
    const double l0 = std::log(1e-6), l1 = std::log(1e4);
    g.r.resize(K);
    g.psi.resize(K);
    for (int i = 0; i < K; i++) g.r[i] = std::exp(l0 + (l1 - l0) * i / (K - 1));
    auto mt = [](double r) { return m_bulge(r) + m_halo(r) + m_disk_sph(r); };
    g.mtot = mt(1e9);
    // psi(r) = int_r^inf M(r') / r'^2 dr' = int M / r d ln r, from the outside in
    g.psi[K - 1] = g.mtot / g.r[K - 1];
    for (int i = K - 2; i >= 0; i--) {
        const double dl = std::log(g.r[i + 1]) - std::log(g.r[i]);
        g.psi[i] = g.psi[i + 1] + 0.5 * dl * (mt(g.r[i]) / g.r[i] + mt(g.r[i + 1]) / g.r[i + 1]);
    }
    return g;
}

// Isotropic distribution function of one spherical component in the total
// potential, tabulated against E = psi(r_j).
struct DF {
    std::vector<double> E, f;            // E decreasing
    double at(double e) const
    {
        if (e <= E.back()) return 0.0;
        if (e >= E.front()) return f.front();
        // E is decreasing: binary search
        size_t lo = 0, hi = E.size() - 1;
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            if (E[mid] > e) lo = mid;
            else hi = mid;
        }
        const double w = (e - E[hi]) / (E[lo] - E[hi]);
        return f[hi] + w * (f[lo] - f[hi]);
    }
};

DF eddington(const Grid &g, double (*rho)(double))
{
    const size_t K = g.r.size();
    std::vector<double> dr(K, 0.0);      // drho/dpsi at grid points
    for (size_t i = 1; i + 1 < K; i++)
        dr[i] = (rho(g.r[i + 1]) - rho(g.r[i - 1])) / (g.psi[i + 1] - g.psi[i - 1]);
    dr[0] = dr[1];
    auto drho_dpsi = [&](double p) -> double {   // interpolation in psi (decreasing with index)
        if (p >= g.psi.front()) return dr.front();
        if (p <= g.psi.back()) return 0.0;
        size_t lo = 0, hi = K - 1;
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            if (g.psi[mid] > p) lo = mid;
            else hi = mid;
        }
        const double w = (p - g.psi[hi]) / (g.psi[lo] - g.psi[hi]);
        return dr[hi] + w * (dr[lo] - dr[hi]);
    };
    // G(E) = int_0^sqrt(E) 2 drho/dpsi(E - t^2) dt  (t = sqrt(E - psi))
    const int J = 1200, T = 400;
    DF d;
    d.E.resize(J);
    std::vector<double> G(J);
    const double e0 = g.psi.front(), e1 = g.psi_at(RV * 1.5);
    for (int j = 0; j < J; j++) {
        const double e = std::exp(std::log(e0) + (std::log(e1) - std::log(e0)) * j / (J - 1));
        d.E[j] = e;
        const double tmax = std::sqrt(e);
        double s = 0.0;
        for (int k = 0; k < T; k++) {
            const double t = tmax * (k + 0.5) / T;
            s += 2.0 * drho_dpsi(e - t * t);
        }
        G[j] = s * tmax / T;
    }
    d.f.resize(J);
    const double norm = 1.0 / (std::sqrt(8.0) * PI * PI);
    for (int j = 0; j < J; j++) {
        const int a = j == 0 ? 0 : j - 1, b = j == J - 1 ? J - 1 : j + 1;
        const double v = (G[a] - G[b]) / (d.E[a] - d.E[b]) * norm;
        d.f[j] = v > 0.0 ? v : 0.0;
    }
    return d;
}

double gauss(Ran3 &r)
{
    // Box-Muller on ran3 uniforms
    const double u1 = r.uniform(1e-300, 1.0), u2 = r.uniform(0.0, 2.0 * PI);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(u2);
}

void iso_direction(Ran3 &r, double len, double *v)
{
    const double ct = r.uniform(-1.0, 1.0), st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    const double ph = r.uniform(0.0, 2.0 * PI);
    v[0] = len * st * std::cos(ph);
    v[1] = len * st * std::sin(ph);
    v[2] = len * ct;
}

// max over v of g(v) = v^2 f(psi - v^2/2) (grid on v = vmax t^2, fine near 0)
double gmax_at(const DF &df, double psi)
{
    const double vmax = std::sqrt(2.0 * psi);
    double m = 0.0;
    const int K = 128;
    for (int k = 1; k < K; k++) {
        const double t = (double)k / K, v = vmax * t * t;
        m = std::max(m, v * v * df.at(psi - 0.5 * v * v));
    }
    return m;
}

// speed at radius r from g(v), by rejection under bound
double sample_speed(Ran3 &r, const DF &df, double psi, double bound)
{
    const double vmax = std::sqrt(2.0 * psi);
    if (!(bound > 0.0)) return 0.0;
    for (int tries = 0; tries < 1000000; tries++) {
        const double v = r.uniform(0.0, vmax);
        if (r.uniform(0.0, bound) <= v * v * df.at(psi - 0.5 * v * v)) return v;
    }
    return 0.0;
}

// radius from a tabulated cumulative mass (monotone), by interpolation
double invert(const std::vector<double> &rr, const std::vector<double> &mm, double u)
{
    const size_t i = std::upper_bound(mm.begin(), mm.end(), u) - mm.begin();
    if (i == 0) return rr.front();
    if (i >= mm.size()) return rr.back();
    const double w = (u - mm[i - 1]) / (mm[i] - mm[i - 1]);
    return rr[i - 1] + w * (rr[i] - rr[i - 1]);
}

}  // namespace

void mkgalaxy(int64_t nd, int64_t nb, int64_t nh, int seed, double *mass, double *phase)
{
    Ran3 r(seed);
    const Grid g = make_grid();
    // ---- disk ----
    {
        const double sigma0 = MD / (2.0 * PI * RD * RD) / (1.0 - (1.0 + RDMAX) * std::exp(-RDMAX));
        std::vector<double> xr(8192), xm(8192);
        for (int k = 0; k < 8192; k++) {
            const double x = RDMAX * k / 8191.0;
            xr[k] = x;
            xm[k] = (1.0 - (1.0 + x) * std::exp(-x)) / (1.0 - (1.0 + RDMAX) * std::exp(-RDMAX));
        }
        auto vc2 = [&](double R) {
            const double y = std::max(R, 1e-8) / (2.0 * RD);
            const double vd2 = 4.0 * PI * sigma0 * RD * y * y *
                               (std::cyl_bessel_i(0.0, y) * std::cyl_bessel_k(0.0, y) -
                                std::cyl_bessel_i(1.0, y) * std::cyl_bessel_k(1.0, y));
            return vd2 + (m_bulge(R) + m_halo(R)) / std::max(R, 1e-8);
        };
        // kinematics on a radius grid (kappa from a centred difference of R^2 vc^2)
        const int KR = 4096;
        std::vector<double> tsr(KR), tsphi(KR), tsz(KR), tvphi(KR);
        for (int k = 0; k < KR; k++) {
            const double R = std::max(RD * RDMAX * k / (KR - 1.0), 1e-4);
            const double h = 1e-3 * R;
            const double v2 = vc2(R), om2 = v2 / (R * R);
            const double L2p = (R + h) * (R + h) * vc2(R + h), L2m = (R - h) * (R - h) * vc2(R - h);
            const double kappa2 = std::max((L2p - L2m) / (2.0 * h) / (R * R * R), 1e-12);
            const double sig = sigma0 * std::exp(-R / RD);
            tsr[k] = QT * 3.36 * sig / std::sqrt(kappa2);
            tsphi[k] = tsr[k] * std::sqrt(kappa2 / (4.0 * om2));
            tsz[k] = std::sqrt(PI * sig * Z0);
            tvphi[k] = std::sqrt(std::max(v2 + tsr[k] * tsr[k] * (1.0 - kappa2 / (4.0 * om2) - 2.0 * R / RD), 0.0));
        }
        auto lerp = [&](const std::vector<double> &t, double R) {
            const double x = R / (RD * RDMAX) * (KR - 1.0);
            const int k = std::min((int)x, KR - 2);
            const double w = x - k;
            return t[k] * (1.0 - w) + t[k + 1] * w;
        };
        for (int64_t i = 0; i < nd; i++) {
            double *p = phase + 6 * i, *v = p + 3;
            mass[i] = MD / (double)nd;
            const double R = RD * invert(xr, xm, r.uniform(0.0, 1.0));
            const double ph = r.uniform(0.0, 2.0 * PI);
            double u = r.uniform(-1.0, 1.0);
            u = std::max(-1.0 + 1e-12, std::min(1.0 - 1e-12, u));
            p[0] = R * std::cos(ph);
            p[1] = R * std::sin(ph);
            p[2] = Z0 * std::atanh(u);
            const double sr = lerp(tsr, R), sphi = lerp(tsphi, R), sz = lerp(tsz, R);
            const double vphi = lerp(tvphi, R) + sphi * gauss(r);
            const double vr = sr * gauss(r), vz = sz * gauss(r);
            v[0] = vr * std::cos(ph) - vphi * std::sin(ph);
            v[1] = vr * std::sin(ph) + vphi * std::cos(ph);
            v[2] = vz;
        }
    }
    // ---- spherical components ----
    auto spherical = [&](int64_t off, int64_t n, double mtot, double (*mfun)(double), double (*rho)(double)) {
        const DF df = eddington(g, rho);
        std::vector<double> rr(8192), mm(8192);
        for (int k = 0; k < 8192; k++) {
            rr[k] = std::exp(std::log(1e-6) + (std::log(RV) - std::log(1e-6)) * k / 8191.0);
            mm[k] = mfun(rr[k]) / mtot;
        }
        // rejection bound per radius: the larger neighbour on the grid, 25% margin
        const int KB = 2048;
        std::vector<double> bnd(KB);
        const double lb0 = std::log(1e-6), lb1 = std::log(RV);
        for (int k = 0; k < KB; k++) bnd[k] = gmax_at(df, g.psi_at(std::exp(lb0 + (lb1 - lb0) * k / (KB - 1.0))));
        for (int64_t i = off; i < off + n; i++) {
            double *p = phase + 6 * i, *v = p + 3;
            mass[i] = mtot / (double)n;
            const double rad = invert(rr, mm, r.uniform(0.0, 1.0));
            iso_direction(r, rad, p);
            const double x = (std::log(std::max(rad, 1e-6)) - lb0) / (lb1 - lb0) * (KB - 1.0);
            const int k = std::max(0, std::min((int)x, KB - 2));
            const double psi = g.psi_at(rad);
            iso_direction(r, sample_speed(r, df, psi, 1.25 * std::max(bnd[k], bnd[k + 1])), v);
        }
    };
    spherical(nd, nb, MB, m_bulge, rho_bulge);
    spherical(nd + nb, nh, MV, m_halo, rho_halo);
    // ---- centre of mass at rest at the origin ----
    const int64_t n = nd + nb + nh;
    double mt = 0.0, cp[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
    for (int64_t i = 0; i < n; i++) {
        mt += mass[i];
        for (int k = 0; k < 3; k++) {
            cp[k] += mass[i] * phase[6 * i + k];
            cv[k] += mass[i] * phase[6 * i + 3 + k];
        }
    }
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            phase[6 * i + k] -= cp[k] / mt;
            phase[6 * i + 3 + k] -= cv[k] / mt;
        }
}

}  // namespace nemo

extern "C" void hc_mkgalaxy(int64_t n_disk, int64_t n_bulge, int64_t n_halo, int seed, double *mass, double *phase)
{
    nemo::mkgalaxy(n_disk, n_bulge, n_halo, seed, mass, phase);
}
