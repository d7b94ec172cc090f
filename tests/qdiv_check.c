/* Checks the FP64 quotient of the exact step (qdiv_rn in fp64_step.cuh): x / d from
 * y = RN(1/d) as q0 = RN(x y), r = fma(-d, q0, x), q = RN(q0 + r y) (q0 for x == 0),
 * bit for bit against IEEE division.  Operands: random significands and exponents,
 * divisors with all-ones significands and near powers of two, signed zeros.
 * Usage: qdiv_check N -> prints "N mismatches", exit status 1 on any. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t state = 0x9E3779B97F4A7C15ULL;
static uint64_t next(void) {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}
static double from_bits(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t to_bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }
static double random_double(int emin, int emax) {
    const uint64_t m = next() & ((1ULL << 52) - 1);
    const int e = emin + (int)(next() % (uint64_t)(emax - emin + 1));
    const double d = from_bits(((uint64_t)(e + 1023) << 52) | m);
    return (next() & 1) ? -d : d;
}
static double qdiv(double x, double d, double y) {
    const double q0 = x * y;
    const double r = fma(-d, q0, x);
    return x == 0.0 ? q0 : fma(r, y, q0);
}
int main(int argc, char **argv) {
    const long n = argc > 1 ? atol(argv[1]) : 1000000L;
    long bad = 0;
    for (long i = 0; i < n; ++i) {
        double x = random_double(-40, 40), d = random_double(-20, 20);
        if (i % 7 == 0) d = from_bits(to_bits(d) | ((1ULL << 52) - 1));
        if (i % 11 == 0) d = from_bits((to_bits(d) & ~((1ULL << 52) - 1)) | (next() & 7));
        if (i % 13 == 0) x = from_bits(to_bits(x) | ((1ULL << 52) - 1));
        if (i % 1009 == 0) x = (i & 1) ? 0.0 : -0.0;
        const double q = qdiv(x, d, 1.0 / d), ref = x / d;
        if (to_bits(q) != to_bits(ref)) {
            if (bad < 5) printf("x=%a d=%a q=%a x/d=%a\n", x, d, q, ref);
            ++bad;
        }
    }
    printf("%ld mismatches\n", bad);
    return bad != 0;
}
