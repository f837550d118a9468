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
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#include "galaxy_model.h"
#include "nemo_io.h"

namespace galaxy {

namespace {

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

// psi(r) = int_r^inf M(r') / r'^2 dr' = int M / r d ln r, from the outside in
void make_grid(Tables &g)
{
    const int K = KG;
    const double l0 = std::log(1e-6), l1 = std::log(1e4);
    g.r.resize(K);
    g.psi.resize(K);
    for (int i = 0; i < K; i++) g.r[i] = std::exp(l0 + (l1 - l0) * i / (K - 1));
    auto mt = [](double r) { return m_bulge(r) + m_halo(r) + m_disk_sph(r); };
    g.mtot = mt(1e9);
    g.psi[K - 1] = g.mtot / g.r[K - 1];
    for (int i = K - 2; i >= 0; i--) {
        const double dl = std::log(g.r[i + 1]) - std::log(g.r[i]);
        g.psi[i] = g.psi[i + 1] + 0.5 * dl * (mt(g.r[i]) / g.r[i] + mt(g.r[i + 1]) / g.r[i + 1]);
    }
}

// Isotropic distribution function of one spherical component in the total
// potential, tabulated against E = psi(r_j) (Eddington's inversion).
void eddington(const Tables &g, const View &gv, double (*rho)(double), std::vector<double> &E,
               std::vector<double> &f)
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
    const int J = JE, T = 400;
    E.resize(J);
    std::vector<double> G(J);
    const double e0 = g.psi.front(), e1 = psi_at(gv, RV * 1.5);
    for (int j = 0; j < J; j++) {
        const double e = std::exp(std::log(e0) + (std::log(e1) - std::log(e0)) * j / (J - 1));
        E[j] = e;
        const double tmax = std::sqrt(e);
        double s = 0.0;
        for (int k = 0; k < T; k++) {
            const double t = tmax * (k + 0.5) / T;
            s += 2.0 * drho_dpsi(e - t * t);
        }
        G[j] = s * tmax / T;
    }
    f.resize(J);
    const double norm = 1.0 / (std::sqrt(8.0) * PI * PI);
    for (int j = 0; j < J; j++) {
        const int a = j == 0 ? 0 : j - 1, b = j == J - 1 ? J - 1 : j + 1;
        const double v = (G[a] - G[b]) / (E[a] - E[b]) * norm;
        f[j] = v > 0.0 ? v : 0.0;
    }
}

// max over v of g(v) = v^2 f(psi - v^2/2) (grid on v = vmax t^2, fine near 0)
double gmax_at(const double *E, const double *f, double psi)
{
    const double vmax = std::sqrt(2.0 * psi);
    double m = 0.0;
    const int K = 128;
    for (int k = 1; k < K; k++) {
        const double t = (double)k / K, v = vmax * t * t;
        m = std::max(m, v * v * df_at(E, f, psi - 0.5 * v * v));
    }
    return m;
}

struct HostDraw {
    nemo::Ran3 &r;
    double operator()(double lo, double hi) { return r.uniform(lo, hi); }
};

}  // namespace

View Tables::view() const
{
    View v{};
    v.r = r.data();
    v.psi = psi.data();
    v.mtot = mtot;
    v.lr0 = r.empty() ? 0.0 : std::log(r.front());
    v.lr1 = r.empty() ? 0.0 : std::log(r.back());
    v.xr = xr.data();
    v.xm = xm.data();
    v.tsr = tsr.data();
    v.tsphi = tsphi.data();
    v.tsz = tsz.data();
    v.tvphi = tvphi.data();
    for (int c = 0; c < 2; c++) {
        v.dfE[c] = dfE[c].data();
        v.dff[c] = dff[c].data();
        v.rr[c] = rr[c].data();
        v.mm[c] = mm[c].data();
        v.bnd[c] = bnd[c].data();
        v.mcomp[c] = mcomp[c];
    }
    return v;
}

void build_tables(Tables &t)
{
    make_grid(t);
    const View gv = t.view();
    // ---- disk: cumulative mass of the truncated exponential, kinematics
    const double sigma0 = MD / (2.0 * PI * RD * RD) / (1.0 - (1.0 + RDMAX) * std::exp(-RDMAX));
    t.xr.resize(NX);
    t.xm.resize(NX);
    for (int k = 0; k < NX; k++) {
        const double x = RDMAX * k / (NX - 1.0);
        t.xr[k] = x;
        t.xm[k] = (1.0 - (1.0 + x) * std::exp(-x)) / (1.0 - (1.0 + RDMAX) * std::exp(-RDMAX));
    }
    auto vc2 = [&](double R) {
        const double y = std::max(R, 1e-8) / (2.0 * RD);
        const double vd2 = 4.0 * PI * sigma0 * RD * y * y *
                           (std::cyl_bessel_i(0.0, y) * std::cyl_bessel_k(0.0, y) -
                            std::cyl_bessel_i(1.0, y) * std::cyl_bessel_k(1.0, y));
        return vd2 + (m_bulge(R) + m_halo(R)) / std::max(R, 1e-8);
    };
    // kinematics on a radius grid (kappa from a centred difference of R^2 vc^2)
    t.tsr.resize(KR);
    t.tsphi.resize(KR);
    t.tsz.resize(KR);
    t.tvphi.resize(KR);
    for (int k = 0; k < KR; k++) {
        const double R = std::max(RD * RDMAX * k / (KR - 1.0), 1e-4);
        const double h = 1e-3 * R;
        const double v2 = vc2(R), om2 = v2 / (R * R);
        const double L2p = (R + h) * (R + h) * vc2(R + h), L2m = (R - h) * (R - h) * vc2(R - h);
        const double kappa2 = std::max((L2p - L2m) / (2.0 * h) / (R * R * R), 1e-12);
        const double sig = sigma0 * std::exp(-R / RD);
        t.tsr[k] = QT * 3.36 * sig / std::sqrt(kappa2);
        t.tsphi[k] = t.tsr[k] * std::sqrt(kappa2 / (4.0 * om2));
        t.tsz[k] = std::sqrt(PI * sig * Z0);
        t.tvphi[k] = std::sqrt(std::max(v2 + t.tsr[k] * t.tsr[k] * (1.0 - kappa2 / (4.0 * om2) - 2.0 * R / RD), 0.0));
    }
    // ---- bulge and halo: distribution functions, mass inversion, bounds
    double (*rho[2])(double) = {rho_bulge, rho_halo};
    double (*mfun[2])(double) = {m_bulge, m_halo};
    for (int c = 0; c < 2; c++) {
        eddington(t, gv, rho[c], t.dfE[c], t.dff[c]);
        t.rr[c].resize(NX);
        t.mm[c].resize(NX);
        for (int k = 0; k < NX; k++) {
            t.rr[c][k] = std::exp(std::log(1e-6) + (std::log(RV) - std::log(1e-6)) * k / (NX - 1.0));
            t.mm[c][k] = mfun[c](t.rr[c][k]) / t.mcomp[c];
        }
        // rejection bound per radius: sampled with the larger grid neighbour and a 25% margin
        t.bnd[c].resize(KB);
        const double lb0 = std::log(1e-6), lb1 = std::log(RV);
        for (int k = 0; k < KB; k++)
            t.bnd[c][k] = gmax_at(t.dfE[c].data(), t.dff[c].data(), psi_at(gv, std::exp(lb0 + (lb1 - lb0) * k / (KB - 1.0))));
    }
}

}  // namespace galaxy

namespace nemo {

void mkgalaxy(int64_t nd, int64_t nb, int64_t nh, int seed, double *mass, double *phase)
{
    using namespace galaxy;
    Ran3 r(seed);
    HostDraw u{r};
    Tables tab;
    build_tables(tab);
    const View t = tab.view();
    bool fail = false;
    for (int64_t i = 0; i < nd; i++) {
        mass[i] = MD / (double)nd;
        disk_body(t, u, phase + 6 * i, phase + 6 * i + 3);
    }
    const int64_t off[2] = {nd, nd + nb}, cnt[2] = {nb, nh};
    for (int c = 0; c < 2; c++)
        for (int64_t i = off[c]; i < off[c] + cnt[c]; i++) {
            mass[i] = t.mcomp[c] / (double)cnt[c];
            sphere_body(t, c, u, phase + 6 * i, phase + 6 * i + 3, &fail);
        }
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
