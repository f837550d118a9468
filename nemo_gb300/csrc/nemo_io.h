// nemo_io.h -- host-side NEMO services for the drop-in programs: the
// portable random generator, the hackcode1 / mkplummer initial conditions,
// the filestruct binary format and the getparam keyword surface.
#pragma once
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

namespace nemo {

// ---- random numbers: NEMO xrandom over NumRec ran3
//      (src/kernel/misc/xrandom.c:90-215, src/kernel/numrec/ran3.c:43-94)
class Ran3 {
public:
    explicit Ran3(int seed = 0) { seed_with(seed); }
    void seed_with(int seed);
    double uniform(double lo, double hi);   // xrandom(lo, hi)
private:
    double next();
    int inext_ = 0, inextp_ = 0, ma_[56] = {0};
};

// hackcode1 nbody= test data (hackcode1/code.c:129-153, util.c:15-27)
void make_testdata(int n, int seed, bool cencon, double *mass, double *phase);
// mkplummer with its defaults (src/nbody/init/mkplummer.c:257-422)
void mkplummer(int n, int seed, double *mass, double *phase);
// isotropic Hernquist sphere (G = M = a = 1) truncated at rtrunc; velocities
// from the Eddington-inverted distribution function (project-written)
void mkhernquist(int n, int seed, double rtrunc, double *mass, double *phase);
// the rejection bound mkhernquist uses: max over v of v^2 f(psi(r) - v^2/2)
// on T radii log-spaced in [exp(lr0), exp(lr1)]
void hernquist_gmax_table(double rtrunc, int T, double *tab, double *lr0, double *lr1);

// ---- filestruct (src/kernel/io/filesecret.c, inc/filestruct.h)
struct Item {
    std::string type;            // "d" "i" "c" "a" "(" ")" ...
    std::string tag;
    std::vector<int> dims;       // empty: singular
    std::vector<unsigned char> data;
    std::vector<Item> items;     // for sets
    const Item *find(const std::string &t) const;
    size_t count() const;        // elements
};

class Writer {
public:
    explicit Writer(FILE *f) : f_(f) {}
    void set(const std::string &tag);
    void tes(const std::string &tag);
    void data(const std::string &tag, const char *type, const void *p, size_t elsize, std::vector<int> dims);
    void string(const std::string &tag, const std::string &s);
    void flush() { fflush(f_); }
private:
    void header(const char *type, const std::string *tag, const std::vector<int> *dims);
    FILE *f_;
};

class Reader {
public:
    explicit Reader(FILE *f) : f_(f) {}
    // next top-level item (a whole set with its contents); false at EOF
    bool next(Item &it);
    bool swapped() const { return swap_; }
private:
    bool read_item(Item &it);
    FILE *f_;
    bool swap_ = false;
};

// snapshot bits (inc/snapshot/snapshot.h)
enum { TimeBit = 1, PhaseSpaceBit = 2, MassBit = 4, PotentialBit = 8, AccelerationBit = 16 };
constexpr int CS_CARTESIAN_3_2 = (1 << 16) | (3 << 8) | 2;   // CSCode(Cartesian, 3, 2)

// Read the next snapshot (get_snap semantics used by hackcode1/hackforce):
// returns false at EOF; throws std::runtime_error on malformed input.
struct Snapshot {
    int nbody = 0;
    double time = 0.0;
    int bits = 0;
    std::vector<double> mass, phase, phi, acc;   // phase [n][2][3], acc [n][3]
};
bool read_snapshot(Reader &r, Snapshot &s, std::vector<std::string> *history = nullptr,
                   std::string *headline = nullptr);
void write_history(Writer &w, const std::vector<std::string> &history, const std::string &headline);

// ---- getparam-style keywords (src/kernel/io/getparam.c)
class Params {
public:
    // defv entries "key=value\n help"; argv[1..] key=value or positional
    Params(const char *const *defv, int argc, char **argv, const char *usage);
    std::string get(const std::string &key) const;
    double getd(const std::string &key) const;       // expressions like 1/32 allowed
    int geti(const std::string &key) const;
    bool getb(const std::string &key) const;
    bool has_value(const std::string &key) const { return !get(key).empty(); }
    const std::string &program() const { return prog_; }
    std::string argv_line() const;
    bool help_requested() const { return help_; }
    // NEMO's debug level: the debug= system keyword, else $DEBUG, else 0
    // (src/kernel/io/getparam.c; dprintf(level, ...) prints when debug >= level)
    int debug_level() const { return debug_; }
private:
    int debug_ = 0;
    std::vector<std::string> keys_;
    std::map<std::string, std::string> vals_;
    std::map<std::string, std::string> helps_;
    std::string prog_, cmdline_;
    bool help_ = false;
};

// scanopt: is word a member of the comma list opts (src/kernel/misc/scanopt.c)
bool scanopt(const std::string &opts, const std::string &word);

// stropen semantics: "-" stdin/stdout, "." /dev/null (src/kernel/io/stropen.c:124-181)
FILE *stropen(const std::string &name, const char *mode);
void strclose(FILE *f);

[[noreturn]] void fatal(const std::string &prog, const std::string &msg);
double cputime_minutes();

}  // namespace nemo
