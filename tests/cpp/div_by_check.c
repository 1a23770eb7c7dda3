/* The FP64 kernels divide the reference's phase numerators by E as
 *     q = x * rE;  q' = fma(fma(-q, E, x), rE, q),   rE = 1/E correctly rounded
 * (Markstein's correction).  This program compares q' with IEEE division x / E on random
 * operands and on operands whose significands sit at the edges (few bits set, nearly all
 * bits set), over exponent ranges wider than the phases' (x = dmv * 2.534 * L, E in GeV).
 * IEEE double arithmetic with a correctly rounded fma behaves identically on the host and
 * the GPU.  Prints the number of mismatches; exit status 1 if there is any. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint64_t next(void) {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}
static double make(uint64_t m, int e, int neg) {
    uint64_t bits = ((uint64_t)(e + 1023) << 52) | (m & ((1ull << 52) - 1));
    if (neg) bits |= 1ull << 63;
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}
static double div_by(double x, double E, double rE) {
    volatile double q = x * rE; /* a separate rounding, as __dmul_rn on the device */
    return fma(fma(-q, E, x), rE, q);
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 20000000;
    long bad = 0;
    for (long i = 0; i < n; i++) {
        const int kind = (int)(i & 3);
        const unsigned k = (unsigned)(next() % 53), j = (unsigned)(next() % 53);
        uint64_t mE = next(), mx = next();
        if (kind == 1) mE = ((1ull << 52) - 1) ^ (next() & ((1ull << k) - 1));
        if (kind == 2) mE = next() & ((1ull << k) - 1);
        if (kind == 3) mx = ((1ull << 52) - 1) ^ (next() & ((1ull << j) - 1));
        const double E = make(mE, (int)(next() % 15) - 7, 0);
        const double x = make(mx, (int)(next() % 41) - 20, (int)(next() & 1));
        const double got = div_by(x, E, 1.0 / E), want = x / E;
        if (got != want) {
            if (bad < 5) printf("x=%a E=%a: %a != %a\n", x, E, got, want);
            bad++;
        }
    }
    printf("%ld pairs, %ld mismatches\n", n, bad);
    return bad ? 1 : 0;
}
