/* Floating-point operation count of the CPU oracle (test infrastructure).
 *
 * The oracle's C sources are compiled a second time, as C++, with `double`
 * replaced by `cfo_counted`: a standard-layout wrapper of one double whose
 * arithmetic operators and math functions count each operation they perform
 * and return the same IEEE result.  The layout is that of a double, so the
 * entry points keep their C-ABI signatures and the ctypes front end calls
 * this library like the plain oracle.  Built serial (no OpenMP) so that the
 * counters are exact; cfo_flops_reset / cfo_flops_read give them to the
 * caller.  Counted: add/subtract, multiply, divide, sqrt, other libm calls
 * (tanh, cosh, pow, exp, log); comparisons, fabs, negation and copies are
 * not arithmetic and are not counted.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stddef.h>

namespace {
unsigned long long n_add, n_mul, n_div, n_sqrt, n_lib;
}

struct cfo_counted {
    double v;
    cfo_counted() = default;
    cfo_counted(double x) : v(x) {}
    explicit operator double() const { return v; }
    cfo_counted &operator+=(cfo_counted o) { ++n_add; v += o.v; return *this; }
    cfo_counted &operator-=(cfo_counted o) { ++n_add; v -= o.v; return *this; }
    cfo_counted &operator*=(cfo_counted o) { ++n_mul; v *= o.v; return *this; }
    cfo_counted &operator/=(cfo_counted o) { ++n_div; v /= o.v; return *this; }
};

static inline cfo_counted operator+(cfo_counted a, cfo_counted b) { ++n_add; return a.v + b.v; }
static inline cfo_counted operator-(cfo_counted a, cfo_counted b) { ++n_add; return a.v - b.v; }
static inline cfo_counted operator*(cfo_counted a, cfo_counted b) { ++n_mul; return a.v * b.v; }
static inline cfo_counted operator/(cfo_counted a, cfo_counted b) { ++n_div; return a.v / b.v; }
static inline cfo_counted operator-(cfo_counted a) { return -a.v; }
static inline cfo_counted operator+(cfo_counted a) { return a; }
static inline bool operator<(cfo_counted a, cfo_counted b) { return a.v < b.v; }
static inline bool operator>(cfo_counted a, cfo_counted b) { return a.v > b.v; }
static inline bool operator<=(cfo_counted a, cfo_counted b) { return a.v <= b.v; }
static inline bool operator>=(cfo_counted a, cfo_counted b) { return a.v >= b.v; }
static inline bool operator==(cfo_counted a, cfo_counted b) { return a.v == b.v; }
static inline bool operator!=(cfo_counted a, cfo_counted b) { return a.v != b.v; }
static inline cfo_counted sqrt(cfo_counted a) { ++n_sqrt; return ::sqrt(a.v); }
static inline cfo_counted fabs(cfo_counted a) { return ::fabs(a.v); }
static inline cfo_counted tanh(cfo_counted a) { ++n_lib; return ::tanh(a.v); }
static inline cfo_counted cosh(cfo_counted a) { ++n_lib; return ::cosh(a.v); }
static inline cfo_counted exp(cfo_counted a) { ++n_lib; return ::exp(a.v); }
static inline cfo_counted log(cfo_counted a) { ++n_lib; return ::log(a.v); }
static inline cfo_counted pow(cfo_counted a, cfo_counted b) { ++n_lib; return ::pow(a.v, b.v); }

static_assert(sizeof(cfo_counted) == sizeof(double), "counted double keeps the layout of a double");

#define double cfo_counted
#include "cf_oracle_flux.c"
#include "cf_oracle_visc.c"
#include "cf_oracle_filter.c"
#include "cf_oracle_lusgs.c"
#undef double

extern "C" {
void cfo_flops_reset(void) { n_add = n_mul = n_div = n_sqrt = n_lib = 0; }
/* add/subtract, multiply, divide, sqrt, other libm calls */
void cfo_flops_read(unsigned long long out[5])
{
    out[0] = n_add; out[1] = n_mul; out[2] = n_div; out[3] = n_sqrt; out[4] = n_lib;
}
}
