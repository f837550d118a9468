/* Checks nemo_gb300/csrc/hc_f32split.h (the build's FP64 -> FP32 rounding and
 * hi + lo splits on a double's bits) against the host's IEEE conversions:
 * random bit patterns, values in the ranges positions and masses take,
 * exact ties of the 29 dropped bits and their neighbours, and the range
 * limits of the integer path.  Exit status 0 when every result matches. */
#include "../../nemo_gb300/csrc/hc_f32split.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

static uint64_t rs = 0x9e3779b97f4a7c15ull;
static uint64_t next(void)
{
    rs ^= rs << 13;
    rs ^= rs >> 7;
    rs ^= rs << 17;
    return rs;
}
static double from_bits(uint64_t u)
{
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
}
static uint32_t fb(float f)
{
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return u;
}

static long checked = 0, bad = 0;
static void check(double x)
{
    if (isnan(x)) return;
    float h, l;
    hc_split_hilo(x, &h, &l);
    const float rh = (float)x, rl = (float)(x - (double)rh), d = hc_d2f_rn(x);
    checked++;
    if (fb(h) != fb(rh) || fb(l) != fb(rl) || fb(d) != fb(rh)) {
        if (bad < 10) printf("mismatch %.17g: hi %08x/%08x lo %08x/%08x rn %08x\n", x, fb(h), fb(rh), fb(l), fb(rl), fb(d));
        bad++;
    }
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    for (long i = 0; i < n; i++) {
        check(from_bits(next()));
        const double u = (double)(next() >> 11) * 0x1p-53 * 8.0 - 4.0;   /* [-4, 4) */
        check(u);
        check(u * 1e-20);
        check(u * 1e30);
        /* ties of the dropped bits and their neighbours */
        uint64_t t = (next() & ~0x1fffffffull) | 0x10000000ull;
        check(from_bits(t));
        check(from_bits(t ^ (1ull << 29)));
        check(from_bits(t + 1));
        check(from_bits(t - 1));
        check(from_bits(t | 0x1fffffffull));
    }
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 1e300, INFINITY, -INFINITY,
                         3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38, 5e-324,
                         0x1p-74, 0x1p-75, -0x1p-74, 0x1p126, 0x1.fffffffffffffp125, -0x1.fffffffffffffp125,
                         0x1.ffffffp0, 0x1.fffffffp0, 0x1.000001p0, 0x1.0000018p0};
    for (size_t i = 0; i < sizeof sp / sizeof sp[0]; i++) check(sp[i]);
    printf("checked %ld, mismatches %ld\n", checked, bad);
    return bad != 0;
}
