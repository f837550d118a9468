// hackcode1 -- drop-in replacement for NEMO's hackcode1 running on the GB300
// library (include/hackcode_gpu.h).
//
// Same keywords, defaults, log table, snapshot stream and state file as
// src/nbody/evolve/hackcode/hackcode1/code.c:21-191 and code_io.c:35-284.
// Documented extensions: usequad= (the hackcode1_qp build), dtime= (sets
// freq = 1/dtime), nstep= (sets tstop = tnow + nstep/freq) and hackcode3's
// potname= / potpars= (an external potential, hackcode3/code.c:136-139).  Interaction
// counts are 64-bit (the reference's int counters wrap near N=1M).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "hackcode_gpu.h"
#include "nemo_io.h"

using namespace nemo;

static const char *defv[] = {
    "in=\n                  snapshot of initial conditions",
    "out=\n                 stream of output snapshots",
    "restart=\n             input state and set controls",
    "continue=\n            input state and continue run",
    "save=\n                output state as code runs",
    "nbody=128\n            number of particles to generate",
    "seed=123\n             random number generator seed",
    "cencon=false\n         centrally concentrated system",
    "freq=32.0\n            fundamental integration frequency",
    "eps=0.05\n             usual potential softening",
    "tol=1.0\n              cell subdivision tolerence",
    "fcells=1.0\n           cell allocation parameter",
    "options=mass,phase\n   misc. control options",
    "tstop=2.0\n            time to stop integration",
    "freqout=4.0\n          major data-output frequency",
    "minor_freqout=32.0\n   minor data-output frequency",
    "log=-\n                logging output",
    "usequad=false\n        quadrupole moments (the hackcode1_qp build)",
    "dtime=\n               time step; sets freq=1/dtime",
    "nstep=\n               number of steps; sets tstop=tnow+nstep/freq",
    "potname=\n             external potential, as hackcode3 (plummer, hernquist, miyamoto, log)",
    "potpars=\n             its parameters, pattern speed first (must be 0)",
    "VERSION=1.5b-gb300\n   GB300 build",
    nullptr,
};

namespace {

struct Run {
    int debug = 0;            // NEMO debug level (debug= / $DEBUG)
    std::string prog, infile, outfile, savefile, options, headline = "Hack code";
    std::vector<std::string> history;
    double freq, eps, tol, fcells, tstop, freqout, minor_freqout, tnow = 0, tout = 0, minor_tout = 0;
    int nstep = 0, nbody = 0;
    bool usequad = false, firstmass = true;
    double rmin[3] = {-2, -2, -2}, rsize = 4;
    std::vector<double> mass, phase, acc, phi;
    hc_ctx *ctx = nullptr;
    FILE *log = nullptr;
    FILE *out = nullptr;
    Writer *w = nullptr;
};

void check(Run &r, int rc, const char *what)
{
    if (rc != HC_OK) fatal(r.prog, std::string(what) + ": " + hc_last_error(r.ctx));
}

// savestate (code_io.c:222-248): the reference's parameter items and the raw
// body table in its in-memory layout (short type, pad, mass, pos, vel, acc,
// phi: 96 bytes per body) so that either program can restart from the file.
void savestate(Run &r, const std::string &file)
{
    FILE *f = stropen(file, "w");
    Writer w(f);
    w.string("program", r.prog);
    w.string("version", "1.5b-gb300");
    w.string("headline", r.headline);
    auto d = [&](const char *tag, double v) { w.data(tag, "d", &v, 8, {}); };
    d("freq", r.freq);
    d("tol", r.tol);
    d("eps", r.eps);
    d("fcells", r.fcells);
    w.string("options", r.options);
    d("tstop", r.tstop);
    d("freqout", r.freqout);
    d("minor_freqout", r.minor_freqout);
    d("tnow", r.tnow);
    d("tout", r.tout);
    d("minor_tout", r.minor_tout);
    w.data("nstep", "i", &r.nstep, 4, {});
    w.data("rmin", "d", r.rmin, 8, {3});
    d("rsize", r.rsize);
    w.data("nbody", "i", &r.nbody, 4, {});
    std::vector<unsigned char> tab((size_t)r.nbody * 96, 0);
    for (int i = 0; i < r.nbody; i++) {
        unsigned char *b = tab.data() + (size_t)96 * i;
        short type = 1;
        memcpy(b, &type, 2);
        memcpy(b + 8, &r.mass[i], 8);
        memcpy(b + 16, &r.phase[6 * i], 24);
        memcpy(b + 40, &r.phase[6 * i + 3], 24);
        memcpy(b + 64, &r.acc[3 * i], 24);
        memcpy(b + 88, &r.phi[i], 8);
    }
    w.data("bodytab", "a", tab.data(), 1, {r.nbody, 96});
    strclose(f);
}

// restorestate (code_io.c:254-284)
void restorestate(Run &r, const std::string &file)
{
    FILE *f = stropen(file, "r");
    Reader rd(f);
    Item it;
    auto need = [&](const Item &x, size_t bytes) {
        if (x.data.size() < bytes) throw std::runtime_error("restorestate: item " + x.tag + " too short in " + file);
    };
    auto getd = [&](const Item &x) {
        double v;
        need(x, 8);
        memcpy(&v, x.data.data(), 8);
        return v;
    };
    auto geti = [&](const Item &x) {
        int v;
        need(x, 4);
        memcpy(&v, x.data.data(), 4);
        return v;
    };
    auto gets = [&](const Item &x) {
        std::string s(x.data.begin(), x.data.end());
        if (!s.empty() && s.back() == 0) s.pop_back();
        return s;
    };
    std::vector<unsigned char> tab;
    while (rd.next(it)) {
        const std::string &t = it.tag;
        if (t == "headline") r.headline = gets(it);
        else if (t == "program") {
            if (gets(it) != r.prog) fprintf(r.log ? r.log : stdout, "warning: state file may be outdated\n\n");
        } else if (t == "freq") r.freq = getd(it);
        else if (t == "tol") r.tol = getd(it);
        else if (t == "eps") r.eps = getd(it);
        else if (t == "fcells") r.fcells = getd(it);
        else if (t == "options") r.options = gets(it);
        else if (t == "tstop") r.tstop = getd(it);
        else if (t == "freqout") r.freqout = getd(it);
        else if (t == "minor_freqout") r.minor_freqout = getd(it);
        else if (t == "tnow") r.tnow = getd(it);
        else if (t == "tout") r.tout = getd(it);
        else if (t == "minor_tout") r.minor_tout = getd(it);
        else if (t == "nstep") r.nstep = geti(it);
        else if (t == "rmin") {
            need(it, 24);
            memcpy(r.rmin, it.data.data(), 24);
        }
        else if (t == "rsize") r.rsize = getd(it);
        else if (t == "nbody") r.nbody = geti(it);
        else if (t == "bodytab") tab = it.data;
    }
    strclose(f);
    if (r.nbody < 1 || tab.size() != (size_t)r.nbody * 96) fatal(r.prog, "restorestate: bad body table in " + file);
    r.mass.assign(r.nbody, 0);
    r.phase.assign(6 * (size_t)r.nbody, 0);
    r.acc.assign(3 * (size_t)r.nbody, 0);
    r.phi.assign(r.nbody, 0);
    for (int i = 0; i < r.nbody; i++) {
        const unsigned char *b = tab.data() + (size_t)96 * i;
        memcpy(&r.mass[i], b + 8, 8);
        memcpy(&r.phase[6 * i], b + 16, 24);
        memcpy(&r.phase[6 * i + 3], b + 40, 24);
        memcpy(&r.acc[3 * i], b + 64, 24);
        memcpy(&r.phi[i], b + 88, 8);
    }
}

// put_snap with the hackcode1 diagnostics set (code_io.c:147-151, 203-216)
void put_snapshot(Run &r, int bits, const hc_diag &d, double cput)
{
    Writer &w = *r.w;
    w.set("SnapShot");
    w.set("Parameters");
    w.data("Nobj", "i", &r.nbody, 4, {});
    if (bits & TimeBit) w.data("Time", "d", &r.tnow, 8, {});
    w.tes("Parameters");
    if (bits & (MassBit | PhaseSpaceBit | PotentialBit | AccelerationBit)) {
        w.set("Particles");
        int cs = CS_CARTESIAN_3_2;
        w.data("CoordSystem", "i", &cs, 4, {});
        if (bits & MassBit) w.data("Mass", "d", r.mass.data(), 8, {r.nbody});
        if (bits & PhaseSpaceBit) w.data("PhaseSpace", "d", r.phase.data(), 8, {r.nbody, 2, 3});
        if (bits & PotentialBit) w.data("Potential", "d", r.phi.data(), 8, {r.nbody});
        if (bits & AccelerationBit) w.data("Acceleration", "d", r.acc.data(), 8, {r.nbody, 3});
        w.tes("Particles");
    }
    w.set("Diagnostics");
    w.data("Energy", "d", d.etot, 8, {3});
    w.data("KETensor", "d", d.keten, 8, {3, 3});
    w.data("PETensor", "d", d.peten, 8, {3, 3});
    w.data("AMTensor", "d", d.amten, 8, {3, 3});
    w.data("CMPhaseSpace", "d", d.cmphase, 8, {2, 3});
    w.data("cputime", "d", &cput, 8, {});
    w.tes("Diagnostics");
    w.tes("SnapShot");
    w.flush();
}

}  // namespace

int main(int argc, char **argv)
{
    Params p(defv, argc, argv, "Barnes & Hut hierarchical N-body tree code (GB300)");
    if (p.help_requested()) return 0;
    Run r;
    r.prog = p.program();
    r.debug = p.debug_level();
    try {
        r.infile = p.get("in");
        r.outfile = p.get("out");
        r.savefile = p.get("save");
        r.options = p.get("options");
        std::string restfile = p.get("restart"), contfile = p.get("continue");
        r.log = stropen(p.get("log"), "w");
        r.usequad = p.getb("usequad");
        if (!contfile.empty()) {
            restorestate(r, contfile);
        } else if (!restfile.empty()) {
            restorestate(r, restfile);
            r.eps = p.getd("eps");          // code.c:93-104
            r.tol = p.getd("tol");
            r.options = p.get("options");
            r.fcells = p.getd("fcells");
            r.tstop = p.getd("tstop");
            r.freqout = p.getd("freqout");
            r.minor_freqout = p.getd("minor_freqout");
            if (scanopt(r.options, "new_tout")) {
                r.tout = r.tnow + 1 / r.freqout;
                r.minor_tout = r.tnow + 1 / r.minor_freqout;
            }
        } else {
            if (!r.infile.empty()) {                  // inputdata, code_io.c:35-56
                FILE *f = stropen(r.infile, "r");
                Reader rd(f);
                Snapshot s;
                if (!read_snapshot(rd, s, &r.history, &r.headline))
                    fatal(r.prog, "inputdata: no snapshot in " + r.infile);
                strclose(f);
                if (!(s.bits & MassBit) || !(s.bits & PhaseSpaceBit)) {
                    char b[96];
                    snprintf(b, sizeof b, "inputdata: essential data missing\tbits = 0x%x", s.bits);
                    fatal(r.prog, b);
                }
                r.nbody = s.nbody;
                r.mass = s.mass;
                r.phase = s.phase;
                r.tnow = ((s.bits & TimeBit) && !scanopt(r.options, "reset_time")) ? s.time : 0.0;
            } else {                                  // make_testdata, code.c:129-153
                r.nbody = p.geti("nbody");
                if (r.nbody < 1) fatal(r.prog, "startrun: absurd nbody");
                r.headline = "Hack code: test data";
                r.mass.assign(r.nbody, 0);
                r.phase.assign(6 * (size_t)r.nbody, 0);
                hc_make_testdata(r.nbody, p.geti("seed"), p.getb("cencon"), r.mass.data(), r.phase.data());
                r.tnow = 0.0;
            }
            r.freq = p.getd("freq");
            if (p.has_value("dtime")) r.freq = 1.0 / p.getd("dtime");
            r.eps = p.getd("eps");
            r.tol = p.getd("tol");
            r.fcells = p.getd("fcells");
            r.tstop = p.getd("tstop");
            if (p.has_value("nstep")) r.tstop = r.tnow + p.geti("nstep") / r.freq;
            r.freqout = p.getd("freqout");
            r.minor_freqout = p.getd("minor_freqout");
            r.nstep = 0;
            r.minor_tout = r.tout = r.tnow;
            r.acc.assign(3 * (size_t)r.nbody, 0);
            r.phi.assign(r.nbody, 0);
        }
    } catch (std::exception &e) {
        fatal(r.prog, e.what());
    }

    hc_params prm{r.tol, r.eps, r.fcells, r.usequad ? 1 : 0, 0};
    if (hc_create(&r.ctx, r.nbody, &prm) != HC_OK) fatal(r.prog, std::string("hc_create: ") + hc_last_error(r.ctx));
    check(r, hc_upload(r.ctx, r.mass.data(), r.phase.data()), "hc_upload");
    check(r, hc_set_box(r.ctx, r.rmin, r.rsize), "hc_set_box");
    check(r, hc_set_forces(r.ctx, r.acc.data(), r.phi.data()), "hc_set_forces");
    if (p.has_value("potname")) {                       // hackcode3 code.c:136-139
        std::vector<double> pars;
        std::string s = p.get("potpars"), item;
        for (size_t i = 0; i <= s.size(); i++) {
            if (i == s.size() || s[i] == ',') {
                if (!item.empty()) {
                    int ok = 0;
                    const double v = hc_nemo_eval(item.c_str(), &ok);
                    if (!ok) fatal(r.prog, "potpars: cannot parse '" + item + "'");
                    pars.push_back(v);
                }
                item.clear();
            } else {
                item += s[i];
            }
        }
        check(r, hc_set_extpot(r.ctx, p.get("potname").c_str(), pars.empty() ? nullptr : pars.data(), (int)pars.size()),
              "hc_set_extpot");
    }

    // initoutput (code_io.c:64-82)
    fprintf(r.log, "\n%s\n\n", r.headline.c_str());
    fprintf(r.log, "%12s%12s%12s%12s\n", "nbody", "freq", "eps", "tol");
    fprintf(r.log, "%12d%12.2f%12.4f%12.4f\n\n", r.nbody, r.freq, r.eps, r.tol);
    if (!r.options.empty()) fprintf(r.log, "\toptions: %s\n", r.options.c_str());
    if (!r.outfile.empty()) {
        r.out = stropen(r.outfile, "w");
        r.w = new Writer(r.out);
        std::vector<std::string> hist = r.history;
        hist.push_back(p.argv_line());
        write_history(*r.w, hist, r.headline);
    }
    if (!r.savefile.empty()) savestate(r, r.savefile);

    double t_gpu = 0;
    long long nbody_steps = 0, ntot = 0;
    while (r.tnow < r.tstop + 0.1 / r.freq) {               // code.c:61
        const double dt = 1.0 / r.freq;
        int bits = 0;                                       // output cadence (code_io.c:130-146)
        if (r.minor_freqout > 0.0 && (r.minor_tout - 0.01 / r.freq) <= r.tnow) {
            r.minor_tout += 1.0 / r.minor_freqout;
            bits |= TimeBit;
        }
        if (r.freqout > 0.0 && (r.tout - 0.01 / r.freq) <= r.tnow) {
            r.tout += 1.0 / r.freqout;
            bits |= TimeBit | PhaseSpaceBit;
            if (scanopt(r.options, "mass") || r.firstmass) {
                bits |= MassBit;
                r.firstmass = false;
            }
            if (scanopt(r.options, "phi")) bits |= PotentialBit;
            if (scanopt(r.options, "acc")) bits |= AccelerationBit;
        }
        bool need = (bits && r.out) || !r.savefile.empty();
        hc_diag d;
        check(r, hc_timer_start(r.ctx), "timer");
        check(r, hc_step(r.ctx, dt, r.nstep, &d, need ? r.phase.data() : nullptr, need ? r.acc.data() : nullptr,
                         need ? r.phi.data() : nullptr),
              "hc_step");
        double ms = 0;
        check(r, hc_timer_stop(r.ctx, &ms), "timer");
        t_gpu += ms;
        nbody_steps += r.nbody;
        ntot += d.n2b + d.nbc;
        const double cput = cputime_minutes();
        long long nttot = d.n2b + d.nbc;
        int nbavg = (int)((double)d.n2b / (double)d.nfcalc), ncavg = (int)((double)d.nbc / (double)d.nfcalc);
        fprintf(r.log, "\n  %10s%10s%10s%10s%10s%10s%10s\n", "tnow", "T+U", "T/U", "nttot", "nbavg", "ncavg", "cputime");
        fprintf(r.log, "  %10.3f%10.4f%10.4f%10lld%10d%10d%10.2f\n\n", r.tnow, d.etot[0], d.etot[1] / d.etot[2], nttot,
                nbavg, ncavg, cput);
        fprintf(r.log, "\t    %10s", "cm pos");
        for (int k = 0; k < 3; k++) fprintf(r.log, "%10.4f", d.cmphase[k]);
        fprintf(r.log, "\n\t    %10s", "cm vel");
        for (int k = 0; k < 3; k++) fprintf(r.log, "%10.4f", d.cmphase[3 + k]);
        fprintf(r.log, "\n");
        if (bits && r.out) {
            put_snapshot(r, bits, d, cput);
            if (bits & PhaseSpaceBit) fprintf(r.log, "\n\tparticle data written\n");
        }
        if (!r.savefile.empty()) {
            check(r, hc_get_box(r.ctx, r.rmin, &r.rsize), "hc_get_box");
            savestate(r, r.savefile);
        }
        r.nstep++;
        r.tnow = r.tnow + dt;
    }
    if (r.out) {
        strclose(r.out);
        delete r.w;
    }
    // the device-time summary goes to stderr at debug >= 1 only (as a dprintf(1, ...)
    // would): the log itself stays the reference's line for line
    if (r.debug >= 1)
        fprintf(stderr, "[%s] gb300: %lld body-steps in %.3f s device time: %.4g bodies/s, %.4g interactions/s\n",
                r.prog.c_str(), nbody_steps, t_gpu * 1e-3, nbody_steps / (t_gpu * 1e-3), ntot / (t_gpu * 1e-3));
    strclose(r.log);
    hc_destroy(r.ctx);
    return 0;
}
