// Host check of the float-float arithmetic used by the MIXFF residual
// (tmp_gb300/csrc/ff_arith.h, the same header the device code includes):
// random operands over twelve decades and both signs, each operation compared
// with the long double result of the operands' exact values.  Prints one line
// per operation: "<op> <max error / bound scale>" where the scale is |exact|
// for *, /, sqrt and |x| + |y| for + and - (the sloppy pair sum is bounded
// relative to its operands).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "../tmp_gb300/csrc/ff_arith.h"

using cfdgb::ff;

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
static double rand_value() {
    const double mag = std::pow(10.0, -6.0 + 12.0 * uniform());
    const double m = 1.0 + uniform();
    return (next_u64() & 1 ? -1.0 : 1.0) * mag * m;
}
static long double exact(ff x) { return (long double)x.hi + (long double)x.lo; }

int main(int argc, char** argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 200000;
    long double e_add = 0, e_sub = 0, e_mul = 0, e_div = 0, e_sqrt = 0, e_canc = 0, e_conv = 0;
    for (int i = 0; i < n; i++) {
        const ff x(rand_value()), y(rand_value());
        const long double X = exact(x), Y = exact(y);
        long double r;
        r = fabsl(exact(x + y) - (X + Y)) / (fabsl(X) + fabsl(Y));
        if (r > e_add) e_add = r;
        r = fabsl(exact(x - y) - (X - Y)) / (fabsl(X) + fabsl(Y));
        if (r > e_sub) e_sub = r;
        r = fabsl(exact(x * y) - X * Y) / fabsl(X * Y);
        if (r > e_mul) e_mul = r;
        r = fabsl(exact(x / y) - X / Y) / fabsl(X / Y);
        if (r > e_div) e_div = r;
        const ff ax = cfdgb::ff_abs(x);
        const long double AX = exact(ax);
        r = fabsl(exact(cfdgb::ff_sqrt(ax)) - sqrtl(AX)) / sqrtl(AX);
        if (r > e_sqrt) e_sqrt = r;
        // near-cancellation: y a relative 1e-9 away from x
        const double xv = (double)x;
        const ff z(xv * (1.0 + 1e-9 * (uniform() - 0.5)));
        const long double Z = exact(z);
        r = fabsl(exact(x - z) - (X - Z)) / (fabsl(X) + fabsl(Z));
        if (r > e_canc) e_canc = r;
        // binary64 -> pair -> binary64
        const double v = rand_value();
        r = fabsl((long double)(double)ff(v) - (long double)v) / fabsl((long double)v);
        if (r > e_conv) e_conv = r;
    }
    std::printf("add %.6Le\nsub %.6Le\nmul %.6Le\ndiv %.6Le\nsqrt %.6Le\ncancel %.6Le\nconvert %.6Le\n", e_add, e_sub,
                e_mul, e_div, e_sqrt, e_canc, e_conv);
    // special values
    const ff zero(0.0), one(1.0);
    std::printf("sqrt0 %g\n", (double)cfdgb::ff_sqrt(zero));
    std::printf("order %d\n", (int)(zero < one && one > zero && !(one < one) && one <= one && -one < zero));
    return 0;
}
