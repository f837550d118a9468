// nemo_io.cpp -- host-side NEMO services for the drop-in programs.
//
//   * xrandom over ran3 and the initial-condition generators used by
//     hackcode1 (nbody=) and by the benchmark workloads (mkplummer),
//   * the filestruct binary format (items, sets, byte-swapped reading),
//   * snapshot read/write in the layout get_snap/put_snap use,
//   * getparam-style keywords with NEMO's system keywords and expressions.
// References are given per function; all code is written for this library.
#include "nemo_io.h"

#include <sys/resource.h>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace nemo {

// ---------------------------------------------------------------- ran3 / xrandom

static const int R3_MBIG = 1000000000, R3_MSEED = 161803398;

// Knuth's subtractive generator as NumRec's ran3 seeds it (ran3.c:43-94);
// set_xrandom(seed > 0) seeds with -seed and discards that first value
// (xrandom.c:147-195).
void Ran3::seed_with(int seed)
{
    int idum = seed > 0 ? -seed : seed;
    int mj = R3_MSEED - (idum < 0 ? -idum : idum);
    while (mj < 0) mj += R3_MBIG;
    mj %= R3_MBIG;
    ma_[55] = mj;
    int mk = 1;
    for (int i = 1; i <= 54; i++) {
        int ii = (21 * i) % 55;
        ma_[ii] = mk;
        mk = mj - mk;
        while (mk < 0) mk += R3_MBIG;
        mj = ma_[ii];
    }
    for (int k = 1; k <= 4; k++)
        for (int i = 1; i <= 55; i++) {
            ma_[i] -= ma_[1 + (i + 30) % 55];
            if (ma_[i] < 0) ma_[i] += R3_MBIG;
        }
    inext_ = 0;
    inextp_ = 31;
    next();   // the seeding call's value is discarded
}

double Ran3::next()
{
    if (++inext_ == 56) inext_ = 1;
    if (++inextp_ == 56) inextp_ = 1;
    int mj = ma_[inext_] - ma_[inextp_];
    while (mj < 0) mj += R3_MBIG;
    ma_[inext_] = mj;
    return mj * (1.0 / R3_MBIG);
}

double Ran3::uniform(double lo, double hi)
{
    if (lo == hi) return lo;
    return lo + next() * (hi - lo);
}

// pickball / pickshell (src/nbody/cores/pickpnt.c:14-48), pickvec (util.c:15-27)
static void pickvec(Ran3 &r, double *v, bool shell)
{
    double rad = shell ? r.uniform(0.0, 1.0) : 1.0;
    double rsq;
    do {
        rsq = 0.0;
        for (int i = 0; i < 3; i++) {
            v[i] = r.uniform(-1.0, 1.0);
            rsq = rsq + v[i] * v[i];
        }
    } while (rsq > 1.0);
    double scale = shell ? rad / std::sqrt(rsq) : rad;
    for (int i = 0; i < 3; i++) v[i] = v[i] * scale;
}

void make_testdata(int n, int seed, bool cencon, double *mass, double *phase)
{
    Ran3 r(seed);
    double cmr[3] = {0, 0, 0}, cmv[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        double *x = phase + 6 * i, *v = x + 3;
        mass[i] = 1.0 / n;
        pickvec(r, x, cencon);
        for (int k = 0; k < 3; k++) cmr[k] = cmr[k] + x[k];
        pickvec(r, v, false);
        for (int k = 0; k < 3; k++) cmv[k] = cmv[k] + v[k];
    }
    for (int k = 0; k < 3; k++) {
        cmr[k] = cmr[k] / (double)n;
        cmv[k] = cmv[k] / (double)n;
    }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            phase[6 * i + k] = phase[6 * i + k] - cmr[k];
            phase[6 * i + 3 + k] = phase[6 * i + 3 + k] - cmv[k];
        }
}

void mkplummer(int n, int seed, double *mass, double *phase)
{
    const double pi = 3.141592653589793238462643, two_pi = 6.283185307179586476925287;
    Ran3 r(seed);
    const double scalefactor = 16.0 / (3.0 * pi);
    const double inv_scale = 1.0 / scalefactor, sqrt_scale = std::sqrt(scalefactor);
    double mfrac = 0.999, rfrac = 22.8042468 * scalefactor;
    double mrfrac = rfrac * rfrac * rfrac / std::pow(1.0 + rfrac * rfrac, 1.5);
    if (mrfrac < mfrac) mfrac = mrfrac;
    double mtot = 0.0;
    for (int i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        mass[i] = 1.0 / (double)n;
        mtot += mass[i];
        double radius = 1.0 / std::sqrt(std::pow(r.uniform(0.0, mfrac), -2.0 / 3.0) - 1.0);
        double theta = std::acos(r.uniform(-1.0, 1.0));
        double phi = r.uniform(0.0, two_pi);
        p[0] = radius * std::sin(theta) * std::cos(phi);
        p[1] = radius * std::sin(theta) * std::sin(phi);
        p[2] = radius * std::cos(theta);
        double x = 0.0, y = 0.1;   // von Neumann rejection for q = v / v_esc
        while (y > x * x * std::pow(1.0 - x * x, 3.5)) {
            x = r.uniform(0.0, 1.0);
            y = r.uniform(0.0, 0.1);
        }
        double velocity = x * std::sqrt(2.0) * std::pow(1.0 + radius * radius, -0.25);
        theta = std::acos(r.uniform(-1.0, 1.0));
        phi = r.uniform(0.0, two_pi);
        v[0] = velocity * std::sin(theta) * std::cos(phi);
        v[1] = velocity * std::sin(theta) * std::sin(phi);
        v[2] = velocity * std::cos(theta);
    }
    for (int i = 0; i < n; i++) {
        mass[i] /= mtot;
        for (int k = 0; k < 3; k++) {
            phase[6 * i + k] = phase[6 * i + k] * inv_scale;
            phase[6 * i + 3 + k] = phase[6 * i + 3 + k] * sqrt_scale;
        }
    }
    double w = 0.0, wp[3] = {0, 0, 0}, wv[3] = {0, 0, 0};
    for (int i = 0; i < n; i++) {
        w = w + 1.0;
        for (int k = 0; k < 3; k++) {
            wp[k] = wp[k] + phase[6 * i + k];
            wv[k] = wv[k] + phase[6 * i + 3 + k];
        }
    }
    for (int k = 0; k < 3; k++) {
        wp[k] = wp[k] / w;
        wv[k] = wv[k] / w;
    }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            phase[6 * i + k] = phase[6 * i + k] - wp[k];
            phase[6 * i + 3 + k] = phase[6 * i + 3 + k] - wv[k];
        }
}

// ---------------------------------------------------------------- Hernquist sphere
//
// Model (Hernquist 1990, ApJ 356, 359), G = M = a = 1:
//   cumulative mass M(r) = r^2 / (1 + r)^2, relative potential psi(r) = 1 / (1 + r),
//   isotropic distribution function of the relative energy E (eq. 17), q = sqrt(E):
//   f(E) = [3 asin q + q sqrt(1 - q^2) (1 - 2 q^2) (8 q^4 - 8 q^2 - 3)]
//          / (8 sqrt(2) pi^3 (1 - q^2)^(5/2)).
// Radii are drawn from M(r) truncated at rtrunc; at radius r the speed has
// density g(v) = v^2 f(psi - v^2 / 2) on [0, sqrt(2 psi)) and is drawn by
// rejection under a tabulated bound of max g (the untruncated potential is
// used for the velocities).  Every body has mass M(rtrunc) / n.  The centre
// of mass and its velocity are removed at the end.

static double hernquist_df(double E)
{
    const double pi = 3.141592653589793238462643;
    if (!(E > 0.0)) return 0.0;
    if (E >= 1.0) E = 1.0 - 1e-15;
    const double q = std::sqrt(E), q2 = E, s = 1.0 - q2;
    const double num = 3.0 * std::asin(q) + q * std::sqrt(s) * (1.0 - 2.0 * q2) * (8.0 * q2 * q2 - 8.0 * q2 - 3.0);
    return num / (8.0 * std::sqrt(2.0) * pi * pi * pi * std::pow(s, 2.5));
}

// max over v of v^2 f(psi - v^2/2): grid on v = vmax t^2 (fine near 0, where
// the peak sits for psi near 1), then golden-section refinement
static double hernquist_gmax(double psi)
{
    const double vmax = std::sqrt(2.0 * psi);
    auto g = [psi](double v) { return v * v * hernquist_df(psi - 0.5 * v * v); };
    const int K = 96;
    int kbest = 0;
    double best = -1.0;
    for (int k = 1; k < K; k++) {
        const double t = (double)k / K, v = vmax * t * t;
        const double y = g(v);
        if (y > best) {
            best = y;
            kbest = k;
        }
    }
    double lo = vmax * std::pow((double)(kbest - 1) / K, 2.0), hi = vmax * std::pow((double)(kbest + 1) / K, 2.0);
    const double gr = 0.6180339887498949;
    for (int it = 0; it < 40; it++) {
        const double a = hi - gr * (hi - lo), b = lo + gr * (hi - lo);
        if (g(a) > g(b)) hi = b;
        else lo = a;
    }
    return std::max(best, g(0.5 * (lo + hi)));
}

void hernquist_gmax_table(double rtrunc, int T, double *tab, double *lr0, double *lr1)
{
    *lr0 = std::log(1e-7);
    *lr1 = std::log(rtrunc * 1.01);
    for (int k = 0; k < T; k++) tab[k] = hernquist_gmax(1.0 / (1.0 + std::exp(*lr0 + (*lr1 - *lr0) * k / (T - 1))));
}

void mkhernquist(int n, int seed, double rtrunc, double *mass, double *phase)
{
    const double two_pi = 6.283185307179586476925287;
    Ran3 r(seed);
    const double mt = rtrunc * rtrunc / ((1.0 + rtrunc) * (1.0 + rtrunc));
    // bound table on log-spaced radii: gmax is smooth in r; use the larger
    // neighbour and a 10% margin
    const int T = 2048;
    double lr0 = 0.0, lr1 = 0.0;
    std::vector<double> tab(T);
    hernquist_gmax_table(rtrunc, T, tab.data(), &lr0, &lr1);
    for (int i = 0; i < n; i++) {
        double *p = phase + 6 * i, *v = p + 3;
        mass[i] = mt / (double)n;
        const double u = std::sqrt(r.uniform(0.0, mt));
        const double radius = u / (1.0 - u);
        double theta = std::acos(r.uniform(-1.0, 1.0));
        double phi = r.uniform(0.0, two_pi);
        p[0] = radius * std::sin(theta) * std::cos(phi);
        p[1] = radius * std::sin(theta) * std::sin(phi);
        p[2] = radius * std::cos(theta);
        const double psi = 1.0 / (1.0 + radius), vesc = std::sqrt(2.0 * psi);
        double x = (std::log(std::max(radius, 1e-7)) - lr0) / (lr1 - lr0) * (T - 1);
        int k = (int)x;
        if (k < 0) k = 0;
        if (k > T - 2) k = T - 2;
        const double bound = 1.1 * std::max(tab[k], tab[k + 1]);
        double speed;
        for (;;) {
            speed = r.uniform(0.0, vesc);
            const double y = r.uniform(0.0, bound);
            if (y <= speed * speed * hernquist_df(psi - 0.5 * speed * speed)) break;
        }
        theta = std::acos(r.uniform(-1.0, 1.0));
        phi = r.uniform(0.0, two_pi);
        v[0] = speed * std::sin(theta) * std::cos(phi);
        v[1] = speed * std::sin(theta) * std::sin(phi);
        v[2] = speed * std::cos(theta);
    }
    double wp[3] = {0, 0, 0}, wv[3] = {0, 0, 0};
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            wp[k] += phase[6 * i + k];
            wv[k] += phase[6 * i + 3 + k];
        }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            phase[6 * i + k] -= wp[k] / n;
            phase[6 * i + 3 + k] -= wv[k] / n;
        }
}

// ---------------------------------------------------------------- filestruct

static const short SING_MAGIC = (011 << 8) + 0222, PLUR_MAGIC = (013 << 8) + 0222;  // filesecret.h:26-27

static size_t type_size(const std::string &t)
{
    switch (t.empty() ? 0 : t[0]) {
    case 'a': case 'c': case 'b': return 1;
    case 's': case 'h': return 2;
    case 'i': case 'f': return 4;
    case 'l': case 'd': return 8;
    default: return 0;
    }
}

const Item *Item::find(const std::string &t) const
{
    for (const Item &i : items)
        if (i.tag == t) return &i;
    return nullptr;
}

size_t Item::count() const
{
    size_t n = 1;
    for (int d : dims) n *= (size_t)d;
    return n;
}

void Writer::header(const char *type, const std::string *tag, const std::vector<int> *dims)
{
    short magic = (dims && !dims->empty()) ? PLUR_MAGIC : SING_MAGIC;
    fwrite(&magic, sizeof magic, 1, f_);
    fwrite(type, 1, strlen(type) + 1, f_);
    if (tag) fwrite(tag->c_str(), 1, tag->size() + 1, f_);
    if (dims && !dims->empty()) {
        fwrite(dims->data(), sizeof(int), dims->size(), f_);
        int z = 0;
        fwrite(&z, sizeof z, 1, f_);
    }
}

void Writer::set(const std::string &tag) { header("(", &tag, nullptr); }
void Writer::tes(const std::string &) { header(")", nullptr, nullptr); }

void Writer::data(const std::string &tag, const char *type, const void *p, size_t elsize, std::vector<int> dims)
{
    header(type, &tag, &dims);
    size_t n = 1;
    for (int d : dims) n *= (size_t)d;
    fwrite(p, elsize, n, f_);
}

void Writer::string(const std::string &tag, const std::string &s)
{
    data(tag, "c", s.c_str(), 1, {(int)s.size() + 1});
}

static void bswap(void *p, size_t size, size_t n)
{
    unsigned char *c = (unsigned char *)p;
    for (size_t i = 0; i < n; i++, c += size)
        for (size_t a = 0, b = size - 1; a < b; a++, b--) std::swap(c[a], c[b]);
}

static bool read_cstr(FILE *f, std::string &s)
{
    s.clear();
    int ch;
    while ((ch = fgetc(f)) != EOF) {
        if (ch == 0) return true;
        s.push_back((char)ch);
    }
    return false;
}

bool Reader::read_item(Item &it)
{
    short magic;
    if (fread(&magic, sizeof magic, 1, f_) != 1) return false;
    bool plural;
    if (magic == SING_MAGIC || magic == PLUR_MAGIC) {
        swap_ = false;
    } else {
        bswap(&magic, sizeof magic, 1);
        if (magic != SING_MAGIC && magic != PLUR_MAGIC) throw std::runtime_error("gethdr: bad magic");
        swap_ = true;
    }
    plural = magic == PLUR_MAGIC;
    if (!read_cstr(f_, it.type)) throw std::runtime_error("gethdr: EOF reading type");
    it.tag.clear();
    if (it.type != ")" && !read_cstr(f_, it.tag)) throw std::runtime_error("gethdr: EOF reading tag");
    it.dims.clear();
    if (plural) {
        for (;;) {
            int d;
            if (fread(&d, sizeof d, 1, f_) != 1) throw std::runtime_error("gethdr: EOF reading dimensions");
            if (swap_) bswap(&d, sizeof d, 1);
            if (d == 0) break;
            if (d < 0) throw std::runtime_error("gethdr: negative dimension " + std::to_string(d));
            it.dims.push_back(d);
        }
    }
    it.items.clear();
    it.data.clear();
    if (it.type == "(") {
        for (;;) {
            Item sub;
            if (!read_item(sub)) throw std::runtime_error("filestruct: EOF inside set " + it.tag);
            if (sub.type == ")") break;
            it.items.push_back(std::move(sub));
        }
    } else if (it.type != ")") {
        size_t es = type_size(it.type);
        if (!es) throw std::runtime_error("filestruct: unknown item type " + it.type);
        size_t n = it.count() * es;
        it.data.resize(n);
        if (n && fread(it.data.data(), 1, n, f_) != n) throw std::runtime_error("filestruct: EOF reading " + it.tag);
        if (swap_ && es > 1) bswap(it.data.data(), es, it.count());
    }
    return true;
}

bool Reader::next(Item &it) { return read_item(it); }

static std::vector<double> as_doubles(const Item &it)
{
    std::vector<double> v(it.count());
    if (it.type == "d") memcpy(v.data(), it.data.data(), v.size() * 8);
    else if (it.type == "f")
        for (size_t i = 0; i < v.size(); i++) {
            float x;
            memcpy(&x, it.data.data() + 4 * i, 4);
            v[i] = x;       // float -> double coercion (filesecret.c copydata_f2d)
        }
    else
        throw std::runtime_error("snapshot: " + it.tag + " is not floating point");
    return v;
}

static int as_int(const Item &it)
{
    int v;
    if (it.type != "i" || it.data.size() < 4) throw std::runtime_error("snapshot: " + it.tag + " is not an int");
    memcpy(&v, it.data.data(), 4);
    return v;
}

bool read_snapshot(Reader &r, Snapshot &s, std::vector<std::string> *history, std::string *headline)
{
    Item it;
    while (r.next(it)) {
        if (it.type == "c" && (it.tag == "History" || it.tag == "Headline")) {
            std::string str(it.data.begin(), it.data.end());
            if (!str.empty() && str.back() == 0) str.pop_back();
            if (it.tag == "History" && history) history->push_back(str);
            if (it.tag == "Headline" && headline) *headline = str;
            continue;
        }
        if (it.type != "(" || it.tag != "SnapShot") continue;
        const Item *par = it.find("Parameters");
        const Item *pts = it.find("Particles");
        if (!par || !pts) continue;            // no particles in this frame
        const Item *nobj = par->find("Nobj");
        if (!nobj) throw std::runtime_error("read_snapshot: Nobj missing");
        s = Snapshot();
        s.nbody = as_int(*nobj);
        if (s.nbody < 1) throw std::runtime_error("read_snapshot: Nobj = " + std::to_string(s.nbody) + " is absurd");
        if (const Item *t = par->find("Time")) {
            const std::vector<double> tv = as_doubles(*t);
            if (tv.empty()) throw std::runtime_error("read_snapshot: Time is empty");
            s.time = tv[0];
            s.bits |= TimeBit;
        }
        if (const Item *cs = pts->find("CoordSystem"))
            if (as_int(*cs) != CS_CARTESIAN_3_2)
                throw std::runtime_error("read_snapshot: cannot handle CoordSystem = " + std::to_string(as_int(*cs)));
        size_t n = (size_t)s.nbody;
        if (const Item *m = pts->find("Mass")) {
            s.mass = as_doubles(*m);
            s.bits |= MassBit;
        }
        if (const Item *p = pts->find("PhaseSpace")) {
            s.phase = as_doubles(*p);
            s.bits |= PhaseSpaceBit;
        } else if (pts->find("Position") && pts->find("Velocity")) {
            std::vector<double> x = as_doubles(*pts->find("Position")), v = as_doubles(*pts->find("Velocity"));
            if (x.size() != 3 * n || v.size() != 3 * n)
                throw std::runtime_error("read_snapshot: Position or Velocity has wrong length");
            s.phase.resize(6 * n);
            for (size_t i = 0; i < n; i++)
                for (int k = 0; k < 3; k++) {
                    s.phase[6 * i + k] = x[3 * i + k];
                    s.phase[6 * i + 3 + k] = v[3 * i + k];
                }
            s.bits |= PhaseSpaceBit;
        }
        if (const Item *p = pts->find("Potential")) {
            s.phi = as_doubles(*p);
            s.bits |= PotentialBit;
        }
        if (const Item *a = pts->find("Acceleration")) {
            s.acc = as_doubles(*a);
            s.bits |= AccelerationBit;
        }
        if ((s.bits & MassBit) && s.mass.size() != n) throw std::runtime_error("read_snapshot: Mass has wrong length");
        if ((s.bits & PhaseSpaceBit) && s.phase.size() != 6 * n)
            throw std::runtime_error("read_snapshot: PhaseSpace has wrong length");
        if ((s.bits & PotentialBit) && s.phi.size() != n)
            throw std::runtime_error("read_snapshot: Potential has wrong length");
        if ((s.bits & AccelerationBit) && s.acc.size() != 3 * n)
            throw std::runtime_error("read_snapshot: Acceleration has wrong length");
        return true;
    }
    return false;
}

void write_history(Writer &w, const std::vector<std::string> &history, const std::string &headline)
{
    if (!headline.empty()) w.string("Headline", headline);
    for (const std::string &h : history) w.string("History", h);
}

// ---------------------------------------------------------------- keywords

namespace {

// Numeric expression evaluator for getdparam (NEMO evaluates "1/32" etc.):
// + - * / ^ **, parentheses, unary signs, pi, sqrt() exp() log() pow(,).
struct Expr {
    const char *p;
    explicit Expr(const char *s) : p(s) {}
    void ws() { while (*p && isspace((unsigned char)*p)) p++; }
    double num()
    {
        ws();
        if (*p == '(') {
            p++;
            double v = sum();
            ws();
            if (*p != ')') throw std::runtime_error("missing )");
            p++;
            return v;
        }
        if (isalpha((unsigned char)*p)) {
            std::string name;
            while (isalnum((unsigned char)*p) || *p == '_') name.push_back(*p++);
            if (name == "pi" || name == "PI") return 3.141592653589793238462643;
            ws();
            if (*p != '(') throw std::runtime_error("unknown name " + name);
            p++;
            double a = sum(), b = 0;
            ws();
            if (*p == ',') {
                p++;
                b = sum();
                ws();
            }
            if (*p != ')') throw std::runtime_error("missing )");
            p++;
            if (name == "sqrt") return std::sqrt(a);
            if (name == "exp") return std::exp(a);
            if (name == "log") return std::log(a);
            if (name == "pow") return std::pow(a, b);
            throw std::runtime_error("unknown function " + name);
        }
        char *end;
        double v = strtod(p, &end);
        if (end == p) throw std::runtime_error("bad number");
        p = end;
        return v;
    }
    double unary()
    {
        ws();
        if (*p == '-') {
            p++;
            return -unary();
        }
        if (*p == '+') {
            p++;
            return unary();
        }
        double b = num();
        ws();
        if (*p == '^' || (p[0] == '*' && p[1] == '*')) {
            p += (*p == '^') ? 1 : 2;
            return std::pow(b, unary());
        }
        return b;
    }
    double prod()
    {
        double v = unary();
        for (;;) {
            ws();
            if (*p == '*' && p[1] != '*') {
                p++;
                v *= unary();
            } else if (*p == '/') {
                p++;
                v /= unary();
            } else
                return v;
        }
    }
    double sum()
    {
        double v = prod();
        for (;;) {
            ws();
            if (*p == '+') {
                p++;
                v += prod();
            } else if (*p == '-') {
                p++;
                v -= prod();
            } else
                return v;
        }
    }
};

const char *SYSTEM_KEYS[] = {"help", "debug", "yapp", "review", "tcl", "error", "outkeys", "np"};

}  // namespace

Params::Params(const char *const *defv, int argc, char **argv, const char *usage)
{
    prog_ = argc > 0 ? argv[0] : "nemo";
    size_t sl = prog_.rfind('/');
    if (sl != std::string::npos) prog_ = prog_.substr(sl + 1);
    for (int i = 0; i < argc; i++) {
        if (i) cmdline_ += " ";
        cmdline_ += argv[i];
    }
    for (int i = 0; defv[i]; i++) {
        std::string e = defv[i];
        size_t nl = e.find('\n');
        std::string kv = e.substr(0, nl), help = nl == std::string::npos ? "" : e.substr(nl + 1);
        size_t eq = kv.find('=');
        std::string k = kv.substr(0, eq), v = eq == std::string::npos ? "" : kv.substr(eq + 1);
        keys_.push_back(k);
        vals_[k] = v;
        helps_[k] = help;
    }
    if (const char *e = getenv("DEBUG")) debug_ = atoi(e);
    std::map<std::string, int> seen;
    bool positional = true;
    size_t posi = 0;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        size_t eq = a.find('=');
        bool named = eq != std::string::npos && eq > 0;
        positional = positional && !named;
        if (positional) {
            if (a == "-help" || a == "--help" || a == "-h" || a == "help") {
                help_ = true;
                continue;
            }
            if (posi >= keys_.size() || keys_[posi] == "VERSION") fatal(prog_, "Too many un-named arguments");
            vals_[keys_[posi]] = a;
            seen[keys_[posi]]++;
            posi++;
            continue;
        }
        if (!named) fatal(prog_, "Arg \"" + a + "\" must be named");
        std::string k = a.substr(0, eq), v = a.substr(eq + 1);
        if (vals_.count(k)) {
            if (seen[k]++) fatal(prog_, "Parameter \"" + k + "\" duplicated");
            vals_[k] = v;
        } else {
            bool sys = false;
            for (const char *s : SYSTEM_KEYS) sys = sys || k == s;
            if (!sys) fatal(prog_, "Parameter \"" + k + "\" unknown");
            if (k == "help") help_ = true;
            if (k == "debug") debug_ = atoi(v.c_str());
        }
    }
    if (help_) {
        printf("%s: %s\n", prog_.c_str(), usage ? usage : "");
        for (const std::string &k : keys_) printf("  %-14s = %-20s %s\n", k.c_str(), vals_[k].c_str(), helps_[k].c_str());
        return;
    }
    for (const std::string &k : keys_)
        if (vals_[k] == "???") fatal(prog_, "Parameter \"" + k + "\" missing");
}

std::string Params::get(const std::string &key) const
{
    auto it = vals_.find(key);
    if (it == vals_.end()) throw std::runtime_error("(getparam) \"" + key + "\" unknown keyword");
    return it->second;
}

double Params::getd(const std::string &key) const
{
    std::string v = get(key);
    try {
        Expr e(v.c_str());
        double r = e.sum();
        e.ws();
        if (*e.p) throw std::runtime_error("trailing characters");
        return r;
    } catch (std::exception &ex) {
        fatal(prog_, "getdparam(" + key + "=" + v + "): " + ex.what());
    }
}

int Params::geti(const std::string &key) const
{
    double d = getd(key);
    return (int)d;
}

bool Params::getb(const std::string &key) const
{
    std::string v = get(key);
    if (v.empty()) fatal(prog_, "getbparam: " + key + "= not bool");
    char c = (char)tolower((unsigned char)v[0]);
    if (c == 't' || c == 'y' || c == '1') return true;
    if (c == 'f' || c == 'n' || c == '0') return false;
    fatal(prog_, "getbparam: " + key + "=" + v + " not bool");
}

std::string Params::argv_line() const { return cmdline_; }

bool scanopt(const std::string &opts, const std::string &word)
{
    size_t i = 0;
    while (i <= opts.size()) {
        size_t j = opts.find(',', i);
        if (j == std::string::npos) j = opts.size();
        std::string w = opts.substr(i, j - i);
        while (!w.empty() && isspace((unsigned char)w.front())) w.erase(w.begin());
        while (!w.empty() && isspace((unsigned char)w.back())) w.pop_back();
        if (w == word) return true;
        i = j + 1;
    }
    return false;
}

FILE *stropen(const std::string &name, const char *mode)
{
    bool write = mode[0] == 'w' || mode[0] == 'a';
    if (name == "-") return write ? stdout : stdin;
    if (name == ".") return fopen("/dev/null", write ? "w" : "r");
    FILE *f = fopen(name.c_str(), mode[0] == 'r' ? "rb" : (mode[0] == 'a' ? "ab" : "wb"));
    if (!f) throw std::runtime_error("stropen: cannot open " + name);
    return f;
}

void strclose(FILE *f)
{
    if (f && f != stdout && f != stdin) fclose(f);
    else if (f) fflush(f);
}

void fatal(const std::string &prog, const std::string &msg)
{
    fflush(stdout);
    fprintf(stderr, "### Fatal error [%s]: %s\n", prog.c_str(), msg.c_str());
    exit(1);
}

double cputime_minutes()
{
    struct rusage ru;
    getrusage(RUSAGE_SELF, &ru);
    return (ru.ru_utime.tv_sec + ru.ru_utime.tv_usec * 1e-6) / 60.0;
}

}  // namespace nemo

using nemo::Expr;

// ---- C entry points for the generators (used by bench.py and the tests)
extern "C" {
// snapcopy: read every snapshot of `in` (with its history) and write it to
// `out` in canonical layout.  Returns the number of snapshots or -1.
int hc_snapcopy(const char *in, const char *out)
{
    FILE *fi = nullptr, *fo = nullptr;
    try {
        fi = nemo::stropen(in, "r");
        nemo::Reader r(fi);
        fo = nemo::stropen(out, "w");
        nemo::Writer w(fo);
        std::vector<std::string> hist;
        std::string head;
        nemo::Snapshot s;
        int count = 0;
        while (nemo::read_snapshot(r, s, &hist, &head)) {
            if (count == 0) nemo::write_history(w, hist, head);
            w.set("SnapShot");
            w.set("Parameters");
            w.data("Nobj", "i", &s.nbody, 4, {});
            if (s.bits & nemo::TimeBit) w.data("Time", "d", &s.time, 8, {});
            w.tes("Parameters");
            w.set("Particles");
            int cs = nemo::CS_CARTESIAN_3_2;
            w.data("CoordSystem", "i", &cs, 4, {});
            if (s.bits & nemo::MassBit) w.data("Mass", "d", s.mass.data(), 8, {s.nbody});
            if (s.bits & nemo::PhaseSpaceBit) w.data("PhaseSpace", "d", s.phase.data(), 8, {s.nbody, 2, 3});
            if (s.bits & nemo::PotentialBit) w.data("Potential", "d", s.phi.data(), 8, {s.nbody});
            if (s.bits & nemo::AccelerationBit) w.data("Acceleration", "d", s.acc.data(), 8, {s.nbody, 3});
            w.tes("Particles");
            w.tes("SnapShot");
            count++;
        }
        nemo::strclose(fi);
        nemo::strclose(fo);
        return count;
    } catch (std::exception &) {
        nemo::strclose(fi);
        nemo::strclose(fo);
        return -1;
    }
}

// getdparam-style expression value (NEMO evaluates e.g. dtime=1/32); *ok = 0 on error
double hc_nemo_eval(const char *expr, int *ok)
{
    try {
        Expr e(expr);
        double v = e.sum();
        e.ws();
        if (*e.p) throw std::runtime_error("trailing characters");
        if (ok) *ok = 1;
        return v;
    } catch (std::exception &) {
        if (ok) *ok = 0;
        return 0.0;
    }
}

void hc_mkplummer(int n, int seed, double *mass, double *phase) { nemo::mkplummer(n, seed, mass, phase); }
void hc_mkhernquist(int n, int seed, double rtrunc, double *mass, double *phase)
{
    nemo::mkhernquist(n, seed, rtrunc, mass, phase);
}
void hc_make_testdata(int n, int seed, int cencon, double *mass, double *phase)
{
    nemo::make_testdata(n, seed, cencon != 0, mass, phase);
}
}
