// hc_gen.cu -- initial conditions drawn on the device, straight into a
// context's body arrays (no counterpart in hackcode1; for systems whose
// generation on the host would take longer than running them).
//
// Models:
//   plummer:   mkplummer's model and sampling steps (src/nbody/init/mkplummer.c,
//              the host restatement in nemo_io.cpp): radius from the cumulative
//              mass inside mfrac, von Neumann rejection for v / v_esc, virial
//              units (16 / 3 pi scaling), equal masses;
//   hernquist: as hc_mkhernquist (truncated sphere, Eddington DF, rejection
//              under the same tabulated bound);
//   galaxy:    as hc_mkgalaxy (disk, bulge, halo): the tables are built on the
//              host by the same code and the per-body steps are the same
//              functions (galaxy_model.h).
// Random numbers: a counter-based stream per body (a 64-bit mixing hash of
// seed, body index and draw number), so every body is drawn independently;
// the draws are not ran3's, so the bodies are a different sample of the same
// model than the host generators give for the same seed.  The centre of mass
// and its velocity are removed at the end (FP64 sums in a fixed order).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "galaxy_model.h"
#include "hc_internal.cuh"
#include "nemo_io.h"

namespace {

constexpr double PI_D = 3.141592653589793238462643;
constexpr int GT = 256, GPART = 304;

__device__ __forceinline__ double urand(uint64_t seed, uint64_t i, uint32_t k)
{
    uint64_t z = seed * 0x9E3779B97F4A7C15ULL ^ (i * 0xBF58476D1CE4E5B9ULL + (uint64_t)k * 0x94D049BB133111EBULL);
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;            // [0, 1)
}

__device__ __forceinline__ void direction(uint64_t seed, uint64_t i, uint32_t k, double len, double *x, double *y,
                                          double *z)
{
    const double ct = 2.0 * urand(seed, i, k) - 1.0, ph = 2.0 * PI_D * urand(seed, i, k + 1);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    *x = len * st * cos(ph);
    *y = len * st * sin(ph);
    *z = len * ct;
}

__global__ void k_gen_plummer(int64_t n, uint64_t seed, double mfrac, double *mass, double *px, double *py,
                              double *pz, double *vx, double *vy, double *vz, int *fails)
{
    const double scale = 16.0 / (3.0 * PI_D), inv = 1.0 / scale, sq = sqrt(scale);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        mass[i] = 1.0 / (double)n;
        const double u = mfrac * fmax(urand(seed, i, 0), 1e-300);
        const double r = 1.0 / sqrt(pow(u, -2.0 / 3.0) - 1.0);
        double x, y, z;
        direction(seed, i, 1, r * inv, &x, &y, &z);
        px[i] = x;
        py[i] = y;
        pz[i] = z;
        double q = 0.0;
        bool ok = false;
        for (uint32_t t = 0; t < 4096 && !ok; t++) {       // von Neumann: q^2 (1 - q^2)^3.5
            q = urand(seed, i, 3 + 2 * t);
            const double yy = 0.1 * urand(seed, i, 4 + 2 * t);
            ok = yy <= q * q * pow(1.0 - q * q, 3.5);
        }
        if (!ok) atomicAdd(fails, 1);
        const double v = q * sqrt(2.0) * pow(1.0 + r * r, -0.25) * sq;
        direction(seed, i, 10000, v, &x, &y, &z);
        vx[i] = x;
        vy[i] = y;
        vz[i] = z;
    }
}

__device__ __forceinline__ double hq_df(double E)
{
    if (!(E > 0.0)) return 0.0;
    if (E >= 1.0) E = 1.0 - 1e-15;
    const double q = sqrt(E), s = 1.0 - E;
    const double num = 3.0 * asin(q) + q * sqrt(s) * (1.0 - 2.0 * E) * (8.0 * E * E - 8.0 * E - 3.0);
    return num / (8.0 * sqrt(2.0) * PI_D * PI_D * PI_D * s * s * sqrt(s));
}

__global__ void k_gen_hernquist(int64_t n, uint64_t seed, double rtrunc, const double *tab, int T, double lr0,
                                double lr1, double *mass, double *px, double *py, double *pz, double *vx,
                                double *vy, double *vz, int *fails)
{
    const double mt = rtrunc * rtrunc / ((1.0 + rtrunc) * (1.0 + rtrunc));
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        mass[i] = mt / (double)n;
        const double u = sqrt(mt * urand(seed, i, 0));
        const double r = u / (1.0 - u);
        double x, y, z;
        direction(seed, i, 1, r, &x, &y, &z);
        px[i] = x;
        py[i] = y;
        pz[i] = z;
        const double psi = 1.0 / (1.0 + r), vesc = sqrt(2.0 * psi);
        const double t = (log(fmax(r, 1e-7)) - lr0) / (lr1 - lr0) * (T - 1);
        int k = (int)t;
        k = k < 0 ? 0 : (k > T - 2 ? T - 2 : k);
        const double bound = 1.1 * fmax(tab[k], tab[k + 1]);
        double v = 0.0;
        bool ok = false;
        for (uint32_t s = 0; s < 65536 && !ok; s++) {
            v = vesc * urand(seed, i, 3 + 2 * s);
            ok = bound * urand(seed, i, 4 + 2 * s) <= v * v * hq_df(psi - 0.5 * v * v);
        }
        if (!ok) atomicAdd(fails, 1);
        direction(seed, i, 200000, v, &x, &y, &z);
        vx[i] = x;
        vy[i] = y;
        vz[i] = z;
    }
}

struct DevDraw {
    uint64_t seed, i;
    uint32_t k;
    __device__ double operator()(double lo, double hi)
    {
        if (lo == hi) return lo;
        return lo + urand(seed, i, k++) * (hi - lo);
    }
};

__global__ void k_gen_galaxy(int64_t n, int64_t nd, int64_t nb, uint64_t seed, galaxy::View t, double *mass,
                             double *px, double *py, double *pz, double *vx, double *vy, double *vz, int *fails)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        DevDraw u{seed, (uint64_t)i, 0};
        double p[3], v[3];
        bool fail = false;
        if (i < nd) {
            mass[i] = galaxy::MD / (double)nd;
            galaxy::disk_body(t, u, p, v);
        } else {
            const int c = i < nd + nb ? 0 : 1;
            mass[i] = t.mcomp[c] / (double)(c == 0 ? nb : n - nd - nb);
            galaxy::sphere_body(t, c, u, p, v, &fail);
        }
        if (fail) atomicAdd(fails, 1);
        px[i] = p[0];
        py[i] = p[1];
        pz[i] = p[2];
        vx[i] = v[0];
        vy[i] = v[1];
        vz[i] = v[2];
    }
}

// the host-built galaxy tables in one device buffer
galaxy::View upload_tables(const galaxy::Tables &t, std::vector<double> &flat, double *dev, size_t *count)
{
    std::vector<std::pair<const std::vector<double> *, const double **>> parts;
    galaxy::View v = t.view();
    parts.push_back({&t.r, &v.r});
    parts.push_back({&t.psi, &v.psi});
    parts.push_back({&t.xr, &v.xr});
    parts.push_back({&t.xm, &v.xm});
    parts.push_back({&t.tsr, &v.tsr});
    parts.push_back({&t.tsphi, &v.tsphi});
    parts.push_back({&t.tsz, &v.tsz});
    parts.push_back({&t.tvphi, &v.tvphi});
    for (int c = 0; c < 2; c++) {
        parts.push_back({&t.dfE[c], &v.dfE[c]});
        parts.push_back({&t.dff[c], &v.dff[c]});
        parts.push_back({&t.rr[c], &v.rr[c]});
        parts.push_back({&t.mm[c], &v.mm[c]});
        parts.push_back({&t.bnd[c], &v.bnd[c]});
    }
    flat.clear();
    for (auto &q : parts) {
        *q.second = dev ? dev + flat.size() : nullptr;
        flat.insert(flat.end(), q.first->begin(), q.first->end());
    }
    *count = flat.size();
    return v;
}

// centre of mass and its velocity: per-block FP64 partials, fixed order
__global__ void __launch_bounds__(GT) k_com_part(int64_t n, const double *m, const double *px, const double *py,
                                                 const double *pz, const double *vx, const double *vy,
                                                 const double *vz, double *part)
{
    __shared__ double sh[7][GT];
    double a[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        a[0] += m[i];
        a[1] += m[i] * px[i];
        a[2] += m[i] * py[i];
        a[3] += m[i] * pz[i];
        a[4] += m[i] * vx[i];
        a[5] += m[i] * vy[i];
        a[6] += m[i] * vz[i];
    }
    for (int q = 0; q < 7; q++) sh[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int o = GT / 2; o; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 7; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 7) part[blockIdx.x * 7 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_com_sub(int64_t n, const double *part, int nb, double *px, double *py, double *pz, double *vx,
                          double *vy, double *vz)
{
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nb; b++)
        for (int q = 0; q < 7; q++) s[q] += part[b * 7 + q];
    const double c[6] = {s[1] / s[0], s[2] / s[0], s[3] / s[0], s[4] / s[0], s[5] / s[0], s[6] / s[0]};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        px[i] -= c[0];
        py[i] -= c[1];
        pz[i] -= c[2];
        vx[i] -= c[3];
        vy[i] -= c[4];
        vz[i] -= c[5];
    }
}

}  // namespace

extern "C" int hc_generate(hc_ctx *c, const char *model, uint64_t seed, const double *par, int npar)
{
    if (!c || !model || npar < 0 || (npar > 0 && !par)) return HC_ERR_ARG;
    const std::string nm = model;
    const int64_t n = c->n;
    int *fails = nullptr;
    double *tab = nullptr;
    struct Release {
        int **f;
        double **t;
        ~Release()
        {
            if (*f) cudaFree(*f);
            if (*t) cudaFree(*t);
        }
    } release{&fails, &tab};
    c->err.clear();
    HC_CUDA(cudaMalloc((void **)&fails, sizeof(int)));
    HC_CUDA(cudaMemsetAsync(fails, 0, sizeof(int), c->stream));
    const int grid = hc_grid(n, GT);
    int r = HC_OK;
    if (nm == "plummer") {
        const double scale = 16.0 / (3.0 * PI_D), rfrac = 22.8042468 * scale;    // mkplummer defaults
        double mfrac = npar > 0 ? par[0] : 0.999;
        const double mr = rfrac * rfrac * rfrac / std::pow(1.0 + rfrac * rfrac, 1.5);
        if (!(mfrac > 0.0) || mfrac > 1.0) r = HC_ERR_ARG;
        if (mr < mfrac) mfrac = mr;
        if (r == HC_OK)
            k_gen_plummer<<<grid, GT, 0, c->stream>>>(n, seed, mfrac, c->mass, c->px, c->py, c->pz, c->vx, c->vy,
                                                      c->vz, fails);
    } else if (nm == "hernquist") {
        const double rt = npar > 0 ? par[0] : 100.0;
        if (!(rt > 0.0)) {
            r = HC_ERR_ARG;
        } else {
            const int T = 2048;
            std::vector<double> h(T);
            double lr0 = 0, lr1 = 0;
            nemo::hernquist_gmax_table(rt, T, h.data(), &lr0, &lr1);
            HC_CUDA(cudaMalloc((void **)&tab, sizeof(double) * T));
            HC_CUDA(cudaMemcpyAsync(tab, h.data(), sizeof(double) * T, cudaMemcpyHostToDevice, c->stream));
            k_gen_hernquist<<<grid, GT, 0, c->stream>>>(n, seed, rt, tab, T, lr0, lr1, c->mass, c->px, c->py, c->pz,
                                                        c->vx, c->vy, c->vz, fails);
        }
    } else if (nm == "galaxy") {
        const int64_t nd = npar > 0 ? (int64_t)par[0] : n / 4, nb = npar > 1 ? (int64_t)par[1] : n / 16;
        if (npar > 2 || nd < 1 || nb < 1 || nd + nb >= n || (npar > 0 && (double)nd != par[0]) ||
            (npar > 1 && (double)nb != par[1])) {
            r = HC_ERR_ARG;
        } else {
            galaxy::Tables t;
            galaxy::build_tables(t);
            std::vector<double> flat;
            size_t cnt = 0;
            upload_tables(t, flat, nullptr, &cnt);
            HC_CUDA(cudaMalloc((void **)&tab, sizeof(double) * cnt));
            const galaxy::View v = upload_tables(t, flat, tab, &cnt);
            HC_CUDA(cudaMemcpyAsync(tab, flat.data(), sizeof(double) * cnt, cudaMemcpyHostToDevice, c->stream));
            k_gen_galaxy<<<grid, GT, 0, c->stream>>>(n, nd, nb, seed, v, c->mass, c->px, c->py, c->pz, c->vx, c->vy,
                                                     c->vz, fails);
            HC_CUDA(cudaStreamSynchronize(c->stream));   // flat is freed on return
        }
    } else {
        c->err = "hc_generate: unknown model '" + nm + "' (plummer, hernquist, galaxy)";
        r = HC_ERR_ARG;
    }
    if (r == HC_OK) {
        const int nb = hc_grid(n, GT, GPART);
        k_com_part<<<nb, GT, 0, c->stream>>>(n, c->mass, c->px, c->py, c->pz, c->vx, c->vy, c->vz, c->diag_part);
        k_com_sub<<<grid, GT, 0, c->stream>>>(n, c->diag_part, nb, c->px, c->py, c->pz, c->vx, c->vy, c->vz);
        double *z[] = {c->ax, c->ay, c->az, c->phi};
        for (double *p : z) HC_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * n, c->stream));
    }
    int nf = 0;
    HC_CUDA(cudaMemcpyAsync(&nf, fails, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    HC_CUDA(cudaGetLastError());
    if (r != HC_OK) {
        if (c->err.empty()) c->err = "hc_generate: bad parameters for '" + nm + "'";
        return r;
    }
    if (nf > 0) {
        c->err = "hc_generate: " + std::to_string(nf) + " velocity draws hit the rejection limit";
        return HC_ERR_STATE;
    }
    c->have_tree = c->have_forces = false;
    return HC_OK;
}
