// hackforce -- drop-in replacement for NEMO's hackforce (one tree force
// evaluation per input snapshot) on the GB300 library.
//
// Keywords, defaults and output layout follow
// src/nbody/evolve/hackcode/hackcode1/hackforce.c:38-272.  Extension:
// usequad= (the hackforce_qp build).  n2btot / nbctot are written as int
// when they fit and as long otherwise (the reference's int wraps near N=1M).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "hackcode_gpu.h"
#include "nemo_io.h"

using namespace nemo;

static const char *defv[] = {
    "in=???\n       Input (snapshot) file with mass coordinates",
    "out=???\n      Output (snapshot) file with f.c. results",
    "test=\n        Input file with test coordinates (if blank, in= coords are used)",
    "tol=1.0\n      Cell subdivision tolerence",
    "eps=0.05\n     Standard softening parameter",
    "rsize=4.0\n    Side-length of initial box",
    "rmin=\n        Lower left corner of initial box [default is -rsize/2 (centered)",
    "options=mass,phase\n Output options: phase and/or mass",
    "fcells=0.75\n  Cell/body allocation ratio",
    "usequad=false\n quadrupole moments (the hackforce_qp build)",
    "VERSION=1.6b-gb300\n GB300 build",
    nullptr,
};

int main(int argc, char **argv)
{
    Params p(defv, argc, argv, "Add hackcode1 computed forces and potential to a snapshot (GB300)");
    if (p.help_requested()) return 0;
    const std::string prog = p.program();
    try {
        const double tol = p.getd("tol"), eps = p.getd("eps"), rsize = p.getd("rsize"), fcells = p.getd("fcells");
        const bool usequad = p.getb("usequad");
        double rmin[3];
        {
            std::vector<double> v;
            std::string s = p.get("rmin");
            for (char &ch : s)
                if (ch == ',') ch = ' ';
            std::istringstream is(s);
            double x;
            while (is >> x) v.push_back(x);
            for (int k = 0; k < 3; k++) rmin[k] = v.size() >= 3 ? v[k] : -rsize / 2.0;   // hackforce.c:187-193
        }
        const std::string options = p.get("options");
        FILE *in = stropen(p.get("in"), "r");
        Reader rin(in);
        FILE *tst = p.has_value("test") ? stropen(p.get("test"), "r") : nullptr;
        Reader *rtest = tst ? new Reader(tst) : nullptr;
        FILE *out = nullptr;
        Writer *w = nullptr;
        std::vector<std::string> history;
        std::string headline;
        Snapshot mass_snap;
        bool have_mass = false;
        for (;;) {
            Snapshot test_snap;
            if (!tst) {                                       // hackforce.c:92-97
                if (!read_snapshot(rin, mass_snap, &history, &headline)) break;
                have_mass = true;
            } else {
                if (!have_mass) {
                    if (!read_snapshot(rin, mass_snap, &history, &headline)) break;
                    have_mass = true;
                }
                if (!read_snapshot(*rtest, test_snap)) break;
            }
            if (!(mass_snap.bits & PhaseSpaceBit) || !(mass_snap.bits & MassBit))
                fatal(prog, "read_snapshot: Mass and PhaseSpace are required");
            const Snapshot &t = tst ? test_snap : mass_snap;
            if (tst && !(t.bits & PhaseSpaceBit)) fatal(prog, "read_snapshot: test positions missing");
            const int nmass = mass_snap.nbody, ntest = t.nbody;
            hc_params prm{tol, eps, fcells, usequad ? 1 : 0, 0};
            hc_ctx *ctx = nullptr;
            if (hc_create(&ctx, nmass, &prm) != HC_OK) fatal(prog, std::string("hc_create: ") + hc_last_error(ctx));
            auto chk = [&](int rc, const char *what) {
                if (rc != HC_OK) fatal(prog, std::string(what) + ": " + hc_last_error(ctx));
            };
            chk(hc_upload(ctx, mass_snap.mass.data(), mass_snap.phase.data()), "hc_upload");
            chk(hc_set_box(ctx, rmin, rsize), "hc_set_box");
            double cputree, cpufcal;
            chk(hc_timer_start(ctx), "timer");
            chk(hc_build_tree(ctx), "maketree");
            chk(hc_timer_stop(ctx, &cputree), "timer");
            std::vector<double> acc(3 * (size_t)ntest), phi(ntest);
            chk(hc_timer_start(ctx), "timer");
            if (!tst) {
                chk(hc_forces(ctx), "hackgrav");
                chk(hc_download(ctx, nullptr, acc.data(), phi.data()), "download");
            } else {
                std::vector<double> tp(3 * (size_t)ntest);
                for (int i = 0; i < ntest; i++)
                    for (int k = 0; k < 3; k++) tp[3 * i + k] = t.phase[6 * i + k];
                chk(hc_forces_at(ctx, tp.data(), ntest, acc.data(), phi.data()), "hackgrav");
            }
            chk(hc_timer_stop(ctx, &cpufcal), "timer");
            hc_diag d;
            chk(hc_diagnostics(ctx, &d), "diagnostics");
            hc_destroy(ctx);

            if (!out) {                                       // out_result, hackforce.c:219-229
                out = stropen(p.get("out"), "w");
                w = new Writer(out);
                history.push_back(p.argv_line());
                write_history(*w, history, headline);
            }
            // write_snapshot, hackforce.c:231-272
            double tsnap = tst ? ((t.bits & TimeBit) ? t.time : 0.0) : mass_snap.time;
            std::vector<double> tmass(ntest, 0.0);
            if (t.bits & MassBit) tmass = t.mass;
            w->set("SnapShot");
            w->set("Parameters");
            w->data("Nobj", "i", &ntest, 4, {});
            w->data("Time", "d", &tsnap, 8, {});
            w->data("tol", "d", &tol, 8, {});
            w->data("eps", "d", &eps, 8, {});
            w->tes("Parameters");
            w->set("Particles");
            int cs = CS_CARTESIAN_3_2;
            w->data("CoordSystem", "i", &cs, 4, {});
            if (scanopt(options, "mass")) w->data("Mass", "d", tmass.data(), 8, {ntest});
            if (scanopt(options, "phase")) w->data("PhaseSpace", "d", t.phase.data(), 8, {ntest, 2, 3});
            w->data("Potential", "d", phi.data(), 8, {ntest});
            w->data("Acceleration", "d", acc.data(), 8, {ntest, 3});
            w->tes("Particles");
            w->set("Diagnostics");
            for (auto [tag, v] : {std::pair<const char *, int64_t>{"n2btot", d.n2b}, {"nbctot", d.nbc}}) {
                if (v <= 2147483647LL) {
                    int iv = (int)v;
                    w->data(tag, "i", &iv, 4, {});
                } else {
                    long lv = (long)v;
                    w->data(tag, "l", &lv, sizeof lv, {});
                }
            }
            double ct = cputree / 60000.0, cf = cpufcal / 60000.0;   // minutes, as cputime() reports
            w->data("cputree", "d", &ct, 8, {});
            w->data("cpufcal", "d", &cf, 8, {});
            w->tes("Diagnostics");
            w->tes("SnapShot");
            w->flush();
        }
        if (out) {
            strclose(out);
            delete w;
        }
        strclose(in);
        if (tst) {
            strclose(tst);
            delete rtest;
        }
    } catch (std::exception &e) {
        fatal(prog, e.what());
    }
    return 0;
}
