// jf_device.cuh -- device arithmetic of the event-time path in FP64 with the reference's semantics.
//
// Compiled with -fmad=false: every FP64 multiply and add is rounded on its own, as CPython rounds Python-level
// float arithmetic and as gcc rounds the reference's C extensions on x86-64.  FMAs appear only where they are
// written out (double-double helpers below).
//
// Reference files (paths relative to the JeLLyFysh source tree):
//   Time ......................... jellyfysh/base/time.py:87-233
//   vectors ...................... jellyfysh/base/vectors.py:30-239
//   periodic boundaries .......... jellyfysh/setting/hypercubic_setting.py:101-172
//   potentials ................... jellyfysh/potential/ (see each function)
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <math_constants.h>

#include "jfgpu.h"

namespace jf {

// The FP64 solve functions of the potentials are out of line by default (small code for kernels that call them from
// many places); a translation unit that defines JF_SOLVE_INLINE inlines them into its callers.
#ifdef JF_SOLVE_INLINE
#define JF_SOLVE __forceinline__
#else
#define JF_SOLVE __noinline__
#endif

constexpr double kInf = __builtin_inf();

__host__ __device__ inline uint64_t double_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof(b));
    return b;
#endif
}

__host__ __device__ inline double bits_double(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
#endif
}

// ---------------------------------------------------------------------------------------------------------------
// CPython float semantics
// ---------------------------------------------------------------------------------------------------------------

// float.__mod__: fmod, then the sign of the divisor (CPython float_rem).
__host__ __device__ inline double py_mod(double x, double y) {
    double mod = fmod(x, y);
    if (mod != 0.0) {
        if ((y < 0.0) != (mod < 0.0)) mod += y;
    } else {
        mod = copysign(0.0, y);
    }
    return mod;
}

// float.__mod__ for x in (-y, 2y), y > 0, without fmod: fmod(x, y) is x for |x| < y and the exact x - y for
// y <= x < 2y; the sign correction of a negative remainder then adds y with one rounding, as CPython does.
__host__ __device__ inline double py_mod_near(double x, double y) {
    // 0 < x < y decided on the bit patterns (positive doubles order as integers; y > 0): no FP64 compare
    const int64_t bx = (int64_t)double_bits(x);
    if (bx > 0 && bx < (int64_t)double_bits(y)) return x;
    if (x == 0.0) return 0.0;
    if (x < 0.0 && x > -y) return x + y;
    if (x >= y && x < 2.0 * y) {
        double r = x - y;
        return r == 0.0 ? 0.0 : r;
    }
    return py_mod(x, y);
}

// divmod(x, 1.0) (CPython float_divmod with the divisor 1.0); fmod(x, 1.0) is the exact x - trunc(x)
__host__ __device__ inline void py_divmod1(double vx, double &quotient, double &remainder) {
    // 0 < vx < 1, decided on the bit pattern: the steps below give (+0.0, vx)
    const int64_t bits = (int64_t)double_bits(vx);
    if (bits > 0 && bits < 0x3FF0000000000000LL) {
        quotient = 0.0;
        remainder = vx;
        return;
    }
    double mod = fabs(vx) < 4503599627370496.0 ? vx - trunc(vx) : fmod(vx, 1.0);
    double div = vx - mod;
    if (mod != 0.0) {
        if (mod < 0.0) {
            mod += 1.0;
            div -= 1.0;
        }
    } else {
        mod = copysign(0.0, 1.0);
    }
    double floordiv;
    if (div != 0.0) {
        floordiv = floor(div);
        if (div - floordiv > 0.5) floordiv += 1.0;
    } else {
        floordiv = copysign(0.0, vx);
    }
    quotient = floordiv;
    remainder = mod;
}

// builtin sum() of three floats from the int 0: the first term exactly, then Neumaier compensation, the
// compensation added at the end when nonzero and finite (CPython 3.12).
__host__ __device__ inline double py_sum3(double a, double b, double c) {
    double f = 0.0 + a;
    double comp = 0.0;
    double t = f + b;
    if (fabs(f) >= fabs(b)) comp += (f - t) + b; else comp += (b - t) + f;
    f = t;
    t = f + c;
    if (fabs(f) >= fabs(c)) comp += (f - t) + c; else comp += (c - t) + f;
    f = t;
    if (comp != 0.0 && isfinite(comp)) f += comp;
    return f;
}

// Time.__add__ (time.py:115-133)
__host__ __device__ inline void time_add(double q, double r, double dt, double &out_q, double &out_r) {
    if (isinf(dt)) {
        out_q = dt;
        out_r = dt;
        return;
    }
    double add_q, new_r;
    py_divmod1(r + dt, add_q, new_r);
    out_q = q + add_q;
    out_r = new_r;
}

// Time.__sub__ (time.py:135-149): left to right
__host__ __device__ inline double time_sub(double q1, double r1, double q2, double r2) { return ((q1 - q2) + r1) - r2; }

// Time.__lt__ (time.py:167-182)
__host__ __device__ inline bool time_lt(double q1, double r1, double q2, double r2) {
    return q1 < q2 || (q1 == q2 && r1 < r2);
}

// ---------------------------------------------------------------------------------------------------------------
// Keyed random numbers: SplitMix64 output function (Steele, Lea and Flood, OOPSLA 2014) on a Weyl state
// key + (counter + 1) * golden, counter = event << 24 | kind << 20 | target.
// ---------------------------------------------------------------------------------------------------------------
constexpr uint64_t kGolden = 0x9e3779b97f4a7c15ULL;

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__host__ __device__ inline uint64_t chain_key(uint64_t seed, uint64_t chain) { return mix64(seed + (chain + 1) * kGolden); }

__host__ __device__ inline uint64_t draw(uint64_t key, uint64_t event, uint32_t kind, uint32_t target) {
    uint64_t counter = (event << 24) | ((uint64_t)(kind & 0xFu) << 20) | (uint64_t)(target & 0xFFFFFu);
    return mix64(key + (counter + 1) * kGolden);
}

enum RngKind : uint32_t { kRngPair = 0, kRngThin = 1, kRngVetoTime = 2, kRngVetoChoice = 3, kRngVetoUniform = 4,
                          kRngNewActive = 5, kRngComposite = 6, kRngLift = 7, kRngCellBound = 8 };

__host__ __device__ inline double uniform53(uint64_t bits) { return (double)(bits >> 11) * (1.0 / 9007199254740992.0); }

__host__ __device__ inline uint32_t randbelow(uint64_t bits, uint32_t n) {
    return (uint32_t)(((bits >> 32) * (uint64_t)n) >> 32);
}

// Natural logarithm written out so that CPU and GPU give the same bits: x = 2^e m, m in [sqrt(1/2), sqrt(2)),
// log m = 2 atanh((m - 1)/(m + 1)) by its Taylor series to the 23rd power (Abramowitz & Stegun 4.1.27).
static __host__ __device__ JF_SOLVE double own_log(double x) {
    uint64_t bits = double_bits(x);
    int e = (int)((bits >> 52) & 0x7FF);
    if (e == 0) {
        x = x * 18014398509481984.0;
        bits = double_bits(x);
        e = (int)((bits >> 52) & 0x7FF) - 54;
    }
    e -= 1023;
    uint64_t mbits = (bits & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL;
    double m = bits_double(mbits);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    double f = (m - 1.0) / (m + 1.0);
    double f2 = f * f;
    double p = 1.0 / 23.0;
    p = p * f2 + 1.0 / 21.0;
    p = p * f2 + 1.0 / 19.0;
    p = p * f2 + 1.0 / 17.0;
    p = p * f2 + 1.0 / 15.0;
    p = p * f2 + 1.0 / 13.0;
    p = p * f2 + 1.0 / 11.0;
    p = p * f2 + 1.0 / 9.0;
    p = p * f2 + 1.0 / 7.0;
    p = p * f2 + 1.0 / 5.0;
    p = p * f2 + 1.0 / 3.0;
    double log_m = 2.0 * f + (2.0 * f) * (f2 * p);
    double de = (double)e;
    const double ln2_hi = 6.93147180369123816490e-01;
    const double ln2_lo = 1.90821492927058770002e-10;
    return de * ln2_hi + (de * ln2_lo + log_m);
}

// random.expovariate(beta) = -log(1.0 - random()) / beta
__host__ __device__ inline double expovariate(uint64_t bits, double beta) { return -own_log(1.0 - uniform53(bits)) / beta; }

// ---------------------------------------------------------------------------------------------------------------
// Powers.  The reference evaluates x ** y with the C library's pow, whose results are correctly rounded in
// all but about 0.1% of cases.  The FP64 path uses correctly rounded powers for the exponents of this path,
// computed in double-double arithmetic (Dekker 1971) with explicit fma, and the CUDA pow otherwise.
// ---------------------------------------------------------------------------------------------------------------
struct DD {
    double hi, lo;
};

__device__ inline DD dd_mul(DD a, DD b) {
    double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e = e + (a.hi * b.lo + a.lo * b.hi);
    double s = p + e;
    return DD{s, e - (s - p)};
}

// x ** n for an integer n >= 1, correctly rounded except in cases within 2^-100 of a rounding boundary
__device__ inline DD dd_ipow(double x, int n) {
    DD result{1.0, 0.0};
    DD base{x, 0.0};
    bool first = true;
    while (n > 0) {
        if (n & 1) {
            result = first ? base : dd_mul(result, base);
            first = false;
        }
        n >>= 1;
        if (n) base = dd_mul(base, base);
    }
    return result;
}

__device__ inline double ipow_cr(double x, int n) {
    if (n == 0) return 1.0;
    double ax = fabs(x);
    if (ax == 0.0 || isinf(ax) || isnan(ax)) return pow(x, (double)n);
    DD r = dd_ipow(ax, n);
    double v = r.hi + r.lo;
    return (x < 0.0 && (n & 1)) ? -v : v;
}

// x ** 1.5 for x >= 0: x * sqrt(x) with the residual of the square root carried in double-double
__device__ inline double pow15_cr(double x) {
    if (!(x > 0.0) || isinf(x)) return pow(x, 1.5);
    double s = sqrt(x);
    double residual = fma(-s, s, x);
    double s_lo = residual / (2.0 * s);
    double p = x * s;
    double p_err = fma(x, s, -p);
    return p + (p_err + x * s_lo);
}

// x ** (1.0 / 6.0) for x > 0 (the exponent is the double nearest 1/6): Newton step on z^6 = x in double-double
// from the CUDA pow, then the correction x^(e - 1/6) = 1 - c log x with c = 1/6 - double(1/6).
static __device__ JF_SOLVE double sixth_root_cr(double x) {
    if (!(x > 1e-30 && x < 1e30)) return pow(x, 1.0 / 6.0);
    // FP32 guess (relative error ~1e-7), one plain Newton step (~1e-14), then the double-double step
    double g = (double)exp2f(__log2f((float)x) * (1.0f / 6.0f));
    double g2 = g * g;
    double g5 = g2 * g2 * g;
    double z0 = g - (g5 * g - x) / (6.0 * g5);
    DD z6 = dd_ipow(z0, 6);
    double residual = (z6.hi - x) + z6.lo;
    double z5 = ipow_cr(z0, 5);
    double dz = residual / (6.0 * z5);
    const double c = 9.25185853854297e-18;
    double lo = -dz - z0 * (c * (double)__logf((float)x));
    return z0 + lo;
}

// Python float ** float on the values of this path: 0 ok, else a JFGPU_STATUS_* code
__device__ inline int py_pow(double x, double y, double &out) {
    if (x < 0.0 && y != floor(y)) return JFGPU_STATUS_COMPLEX;
    if (x == 0.0 && y < 0.0) return JFGPU_STATUS_ZERO_DIVISION;
    if (y == 2.0) {
        out = x * x;
    } else if (y == 0.5) {
        out = sqrt(x);
    } else if (y == 1.5) {
        out = pow15_cr(x);
    } else if (y == 1.0 / 6.0) {
        out = sixth_root_cr(x);
    } else if (y == floor(y) && fabs(y) <= 64.0 && y > 0.0) {
        out = ipow_cr(x, (int)y);
    } else {
        out = pow(x, y);
    }
    return JFGPU_STATUS_OK;
}

#define JF_DIV(a, b, out)                                                                                          \
    do {                                                                                                           \
        double divisor_ = (b);                                                                                     \
        if (divisor_ == 0.0) return JFGPU_STATUS_ZERO_DIVISION;                                                    \
        (out) = (a) / divisor_;                                                                                    \
    } while (0)
#define JF_TRY(expr)                                                                                               \
    do {                                                                                                           \
        int status_ = (expr);                                                                                      \
        if (status_) return status_;                                                                               \
    } while (0)

// ---------------------------------------------------------------------------------------------------------------
// vectors (base/vectors.py)
// ---------------------------------------------------------------------------------------------------------------
__device__ inline double norm_sq3(const double *v) { return py_sum3(v[0] * v[0], v[1] * v[1], v[2] * v[2]); }

__device__ inline double norm3(const double *v) { return sqrt(norm_sq3(v)); }  // sum(...) ** 0.5

// sum([value ** 2 for value of the other components]) (vectors.py:181, 213); two terms sum plainly
__device__ inline double perp_sq(const double *v, int d) {
    int a = d == 0 ? 1 : 0;
    int b = d == 2 ? 1 : 2;
    return (0.0 + v[a] * v[a]) + v[b] * v[b];
}

// displacement_until_new_norm_sq_component_positive (vectors.py:153-181)
__device__ inline int disp_until_positive(const double *v, double norm_sq_new, int d, double &out) {
    if (!(v[d] > 0.0)) return JFGPU_STATUS_ASSERTION;
    double radicand = norm_sq_new - perp_sq(v, d);
    if (radicand < 0.0) return JFGPU_STATUS_VALUE_ERROR;
    out = v[d] - sqrt(radicand);
    return JFGPU_STATUS_OK;
}

// displacement_until_new_norm_sq_component_negative (vectors.py:184-214)
__device__ inline int disp_until_negative(const double *v, double norm_sq_new, int d, double &out) {
    if (!(v[d] <= 0.0)) return JFGPU_STATUS_ASSERTION;
    double radicand = norm_sq_new - perp_sq(v, d);
    if (radicand < 0.0) return JFGPU_STATUS_VALUE_ERROR;
    out = v[d] + sqrt(radicand);
    return JFGPU_STATUS_OK;
}

// StandardVelocityPotential._analyse_velocity (potential/abstracts.py:115-140)
__device__ inline int analyse_velocity(const double *velocity, int &direction, double &speed) {
    int count = 0, dir = -1;
    for (int i = 0; i < 3; ++i)
        if (velocity[i] != 0.0) {
            ++count;
            dir = i;
        }
    if (count != 1 || !(velocity[dir] > 0.0)) return JFGPU_STATUS_ASSERTION;
    direction = dir;
    speed = velocity[dir];
    return JFGPU_STATUS_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Hard sphere (potential/hard_sphere_potential.py:65-99)
// ---------------------------------------------------------------------------------------------------------------
__device__ inline int hs_displacement(double diameter_squared, const double *velocity, const double *s, double &out) {
    double velocity_squared = norm_sq3(velocity);
    if (!(velocity_squared > 0.0)) return JFGPU_STATUS_ASSERTION;
    double separation_squared = norm_sq3(s);
    if (!(separation_squared - diameter_squared > -1.0e-13)) return JFGPU_STATUS_ASSERTION;
    double vds = py_sum3(velocity[0] * s[0], velocity[1] * s[1], velocity[2] * s[2]);
    double square_root_term = vds * vds - velocity_squared * (separation_squared - diameter_squared);
    out = (square_root_term >= 0.0 && vds >= 0.0) ? (vds - sqrt(square_root_term)) / velocity_squared : kInf;
    return JFGPU_STATUS_OK;
}

// Hard sphere with an axis-aligned positive velocity of the given speed (the event loop's form): the sums of
// the velocity products collapse to their single nonzero term exactly.
__device__ inline int hs_displacement_axis(double diameter_squared, int d, double speed, const double *s, double &out) {
    double velocity[3] = {0.0, 0.0, 0.0};
    velocity[d] = speed;
    return hs_displacement(diameter_squared, velocity, s, out);
}

// ---------------------------------------------------------------------------------------------------------------
// Inverse power potential (potential/inverse_power_potential.py)
// ---------------------------------------------------------------------------------------------------------------
struct IP {
    double power, prefactor, two_over_power, power_over_two, power_plus_two;
};

__host__ __device__ inline IP ip_make(double power, double prefactor) {
    IP p;
    p.power = power;
    p.prefactor = prefactor;
    p.two_over_power = 2.0 / power;
    p.power_over_two = power / 2.0;
    p.power_plus_two = power + 2.0;
    return p;
}

__device__ inline int ip_potential(const IP &p, double cp, const double *s, double &out) {  // :127-143
    double denominator;
    JF_TRY(py_pow(norm_sq3(s), p.power_over_two, denominator));
    JF_DIV(cp * p.prefactor, denominator, out);
    return JFGPU_STATUS_OK;
}

__device__ inline int ip_std_derivative(const IP &p, int d, const double *s, double c1, double c2, double &out) {
    double denominator, value;  // :71-94
    JF_TRY(py_pow(norm3(s), p.power_plus_two, denominator));
    JF_DIV(p.power * s[d], denominator, value);
    out = ((value * p.prefactor) * c1) * c2;
    return JFGPU_STATUS_OK;
}

__device__ inline int ip_std_displacement(const IP &p, int d, double *s, double c1, double c2, double du, double &out) {
    double cp = c1 * c2;
    if (p.prefactor * cp > 0.0) {  // _displacement_repulsive (:145-161)
        if (s[d] <= 0.0) {
            out = kInf;
            return JFGPU_STATUS_OK;
        }
        double s_max[3] = {s[0], s[1], s[2]};
        s_max[d] = 0.0;
        double maximum_potential, current_potential;
        JF_TRY(ip_potential(p, cp, s_max, maximum_potential));
        JF_TRY(ip_potential(p, cp, s, current_potential));
        if (du < maximum_potential - current_potential) {
            double ratio, nsq;
            JF_DIV(cp * p.prefactor, current_potential + du, ratio);
            JF_TRY(py_pow(ratio, p.two_over_power, nsq));
            return disp_until_positive(s, nsq, d, out);
        }
        out = kInf;
        return JFGPU_STATUS_OK;
    }
    double displacement = 0.0;  // _displacement_attractive (:163-179)
    if (s[d] > 0.0) {
        displacement += s[d];
        s[d] = 0.0;
    }
    double current_potential;
    JF_TRY(ip_potential(p, cp, s, current_potential));
    if (current_potential + du >= 0.0) {
        out = kInf;
        return JFGPU_STATUS_OK;
    }
    double ratio, nsq, extra;
    JF_DIV(cp * p.prefactor, current_potential + du, ratio);
    JF_TRY(py_pow(ratio, p.two_over_power, nsq));
    JF_TRY(disp_until_negative(s, nsq, d, extra));
    out = displacement + extra;
    return JFGPU_STATUS_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Mexican-hat potentials (potential/abstracts.py:336-530): Lennard-Jones (lennard_jones_potential.py) and
// displaced even power (displaced_even_power_potential.py).  Host code fills the constants with the host's pow
// so that r0 = sigma * 2 ** (1 / 6) and the prefactors equal the reference's.
// ---------------------------------------------------------------------------------------------------------------
struct MH {
    int kind;  // 0 Lennard-Jones, 1 displaced even power
    double prefactor, r0, r0_squared;
    double sigma;
    IP six, twelve;
    double power, inverse_power;
};

// Lennard-Jones potential six.potential(1, s) + twelve.potential(1, s) (lennard_jones_potential.py:83-98,
// inverse_power_potential.py:127-143): k sigma^6 / |s|^6 terms from norm_sq ** 3.0 and norm_sq ** 6.0, both
// correctly rounded from one double-double cube
static __device__ JF_SOLVE int lj_potential(const MH &h, const double *s, double &out) {
    double ns = norm_sq3(s);
    if (!(ns > 0.0) || isinf(ns)) {
        double a, b;
        JF_TRY(ip_potential(h.six, 1.0, s, a));
        JF_TRY(ip_potential(h.twelve, 1.0, s, b));
        out = a + b;
        return JFGPU_STATUS_OK;
    }
    DD n3 = dd_ipow(ns, 3);
    DD n6 = dd_mul(n3, n3);
    double p3 = n3.hi + n3.lo;
    double p6 = n6.hi + n6.lo;
    double a, b;
    JF_DIV(1.0 * h.six.prefactor, p3, a);
    JF_DIV(1.0 * h.twelve.prefactor, p6, b);
    out = a + b;
    return JFGPU_STATUS_OK;
}

__device__ inline int mh_potential(const MH &h, const double *s, double &out) {
    if (h.kind == 0) return lj_potential(h, s, out);
    double powered;
    JF_TRY(py_pow(norm3(s) - h.r0, h.power, powered));
    out = h.prefactor * powered;
    return JFGPU_STATUS_OK;
}

static __device__ JF_SOLVE int mh_invert_inside(const MH &h, double potential, double &out) {
    if (h.kind == 0) {  // lennard_jones_potential.py:100-115
        double root, denominator;
        JF_TRY(py_pow(1.0 + (4.0 * potential) / h.prefactor, 0.5, root));
        JF_TRY(py_pow((1.0 + root) / 2.0, 1.0 / 6.0, denominator));
        JF_DIV(h.sigma, denominator, out);
        return JFGPU_STATUS_OK;
    }
    double powered;
    JF_TRY(py_pow(potential / h.prefactor, h.inverse_power, powered));
    out = h.r0 - powered;
    return JFGPU_STATUS_OK;
}

static __device__ JF_SOLVE int mh_invert_outside(const MH &h, double potential, double &out) {
    if (h.kind == 0) {  // lennard_jones_potential.py:117-135
        if (potential >= 0.0) {
            out = kInf;
            return JFGPU_STATUS_OK;
        }
        double root, denominator;
        JF_TRY(py_pow(1.0 + (4.0 * potential) / h.prefactor, 0.5, root));
        JF_TRY(py_pow((1.0 - root) / 2.0, 1.0 / 6.0, denominator));
        JF_DIV(h.sigma, denominator, out);
        return JFGPU_STATUS_OK;
    }
    double powered;
    JF_TRY(py_pow(potential / h.prefactor, h.inverse_power, powered));
    out = h.r0 + powered;
    return JFGPU_STATUS_OK;
}

static __device__ JF_SOLVE int mh_front_outside(const MH &h, int d, double u, double du, double *s, double &out) {
    double norm_new;  // abstracts.py:384-408
    JF_TRY(mh_invert_outside(h, u + du, norm_new));
    return disp_until_negative(s, norm_new * norm_new, d, out);
}

static __device__ JF_SOLVE int mh_front_inside(const MH &h, int d, double du, double *s, double &out) {
    double displacement, u, extra;  // abstracts.py:456-484
    JF_TRY(disp_until_negative(s, h.r0_squared, d, displacement));
    s[d] -= displacement;
    JF_TRY(mh_potential(h, s, u));
    JF_TRY(mh_front_outside(h, d, u, du, s, extra));
    out = displacement + extra;
    return JFGPU_STATUS_OK;
}

static __device__ JF_SOLVE int mh_behind_inside(const MH &h, int d, double u, double du, double *s, double &out) {
    double s_max[3] = {s[0], s[1], s[2]};  // abstracts.py:486-530
    s_max[d] = 0.0;
    double u_max;
    JF_TRY(mh_potential(h, s_max, u_max));
    double difference = u_max - u;
    if (du < difference) {
        double norm_new;
        JF_TRY(mh_invert_inside(h, u + du, norm_new));
        return disp_until_positive(s, norm_new * norm_new, d, out);
    }
    double displacement = s[d];
    s[d] = 0.0;
    du -= difference;
    double extra;
    JF_TRY(mh_front_inside(h, d, du, s, extra));
    out = displacement + extra;
    return JFGPU_STATUS_OK;
}

// abstracts.py:410-454: a ValueError anywhere in the try block switches to the fallback, which sees the
// separation as mutated up to that point
static __device__ JF_SOLVE int mh_behind_outside(const MH &h, int d, double du, double *s, double &out) {
    double displacement, u, extra;
    int st = disp_until_positive(s, h.r0_squared, d, displacement);
    if (st == JFGPU_STATUS_OK) {
        s[d] -= displacement;
        st = mh_potential(h, s, u);
        if (st == JFGPU_STATUS_OK) {
            st = mh_behind_inside(h, d, u, du, s, extra);
            if (st == JFGPU_STATUS_OK) {
                out = displacement + extra;
                return JFGPU_STATUS_OK;
            }
        }
    }
    if (st != JFGPU_STATUS_VALUE_ERROR) return st;
    displacement = s[d];
    s[d] = 0.0;
    JF_TRY(mh_potential(h, s, u));
    JF_TRY(mh_front_outside(h, d, u, du, s, extra));
    out = displacement + extra;
    return JFGPU_STATUS_OK;
}

// MexicanHatPotential.standard_velocity_displacement (abstracts.py:336-382); s is mutated
__device__ inline int mh_std_displacement(const MH &h, int d, double *s, double du, double &out) {
    double norm = norm3(s);
    if (norm >= h.r0) {
        if (s[d] <= 0.0) {
            double u;
            JF_TRY(mh_potential(h, s, u));
            return mh_front_outside(h, d, u, du, s, out);
        }
        return mh_behind_outside(h, d, du, s, out);
    }
    if (s[d] <= 0.0) return mh_front_inside(h, d, du, s, out);
    double u;
    JF_TRY(mh_potential(h, s, u));
    return mh_behind_inside(h, d, u, du, s, out);
}

// Lennard-Jones space derivative (lennard_jones_potential.py:63-81 with inverse_power_potential.py:71-94):
// norm ** 8 and norm ** 14 correctly rounded from shared double-double powers
static __device__ JF_SOLVE int lj_std_derivative(const MH &h, int d, const double *s, double &out) {
    double n = norm3(s);
    if (!(n > 0.0) || isinf(n)) {
        double a, b;
        JF_TRY(ip_std_derivative(h.six, d, s, 1.0, 1.0, a));
        JF_TRY(ip_std_derivative(h.twelve, d, s, 1.0, 1.0, b));
        out = a + b;
        return JFGPU_STATUS_OK;
    }
    DD n2 = dd_mul(DD{n, 0.0}, DD{n, 0.0});
    DD n4 = dd_mul(n2, n2);
    DD n8 = dd_mul(n4, n4);
    DD n14 = dd_mul(dd_mul(n8, n4), n2);
    double p8 = n8.hi + n8.lo;
    double p14 = n14.hi + n14.lo;
    double a, b;
    JF_DIV(h.six.power * s[d], p8, a);
    JF_DIV(h.twelve.power * s[d], p14, b);
    out = ((a * h.six.prefactor) * 1.0) * 1.0 + ((b * h.twelve.prefactor) * 1.0) * 1.0;
    return JFGPU_STATUS_OK;
}

__device__ inline int mh_std_derivative(const MH &h, int d, const double *s, double &out) {
    if (h.kind == 0) return lj_std_derivative(h, d, s, out);
    double norm = norm3(s);  // displaced_even_power_potential.py:73-93
    double powered;
    JF_TRY(py_pow(norm - h.r0, h.power - 1.0, powered));
    JF_DIV((((-h.power) * h.prefactor) * powered) * s[d], norm, out);
    return JFGPU_STATUS_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// Inverse-power Coulomb bounding potential
// (inverse_power_coulomb_bounding_potential.c:53-139; the Python wrapper permutes the separation so that the
//  motion axis comes first, vectors.py:220-239)
// ---------------------------------------------------------------------------------------------------------------
__device__ inline void permute3(const double *s, int d, double *p) {
    p[0] = s[d];
    p[1] = s[d == 2 ? 0 : d + 1];
    p[2] = s[d == 0 ? 2 : d - 1];
}

__device__ inline double ipcb_x_derivative(double pp, double sx, double sy, double sz) {
    return pp * sx / pow15_cr(sx * sx + sy * sy + sz * sz);
}

__device__ inline double ipcb_potential(double pp, double sx, double sy, double sz) {
    return pp / sqrt(sx * sx + sy * sy + sz * sz);
}

static __device__ __noinline__ double ipcb_x_displacement(double pp, double sx, double sy, double sz, double du, double length) {
    double half = length / 2.0;
    double current = ipcb_potential(pp, sx, sy, sz);
    double u_zero = ipcb_potential(pp, 0.0, sy, sz);
    double u_half = ipcb_potential(pp, half, sy, sz);
    double per_length = fabs(u_zero - u_half);
    double displacement;
    if (du >= 0.0 && du < per_length * (1.0 - 0x1p-50)) {
        // floor(du / per_length) is 0 (the product's rounding keeps du below per_length (1 - 2^-51), so the rounded
        // quotient stays below 1) and fmod returns du itself: the same values without the division and fmod
        displacement = 0.0 * length;
    } else {
        displacement = floor(du / per_length) * length;
        du = fmod(du, per_length);
    }
    double new_norm;
    if (pp > 0.0) {
        if (sx <= 0.0) {
            displacement += half + sx;
            sx = half;
            current = u_half;
        } else if (du >= u_zero - current) {
            du -= (u_zero - current);
            displacement += sx + half;
            sx = half;
            current = u_half;
        }
        new_norm = pp / (current + du);
        displacement += (sx - sqrt(new_norm * new_norm - (sy * sy + sz * sz)));
    } else {
        if (sx > 0.0) {
            displacement += sx;
            sx = 0.0;
            current = u_zero;
        } else if (du >= u_half - current) {
            du -= (u_half - current);
            displacement += sx + length;
            sx = 0.0;
            current = u_zero;
        }
        new_norm = pp / (current + du);
        displacement += (sx + sqrt(new_norm * new_norm - (sy * sy + sz * sz)));
    }
    return displacement;
}

// ---------------------------------------------------------------------------------------------------------------
// Merged-image Coulomb potential: x-derivative of the Ewald sum
// (merged_image_coulomb_potential.c:205-274; Fourier coefficients built on the host, :77-119)
// ---------------------------------------------------------------------------------------------------------------
struct MIC {
    int fourier_cutoff, fourier_cutoff_sq, position_cutoff, position_cutoff_sq;
    double alpha_over_length, alpha_over_length_sq, two_alpha_over_length_root_pi, system_length, two_pi_over_length;
    const double *fourier;  // [(fc+1)^3] index (i*(fc+1)+j)*(fc+1)+k
};

static __device__ __noinline__ double mic_x(const MIC &m, double sx, double sy, double sz) {
    double derivative = 0.0;
    int n = m.fourier_cutoff + 1;
    for (int k = -m.position_cutoff; k < m.position_cutoff + 1; k++) {
        double vector_z_sq = (sz + k * m.system_length) * (sz + k * m.system_length);
        int cutoff_y = (int)sqrt((double)(m.position_cutoff_sq - k * k));
        for (int j = -cutoff_y; j < cutoff_y + 1; j++) {
            double vector_y_sq = (sy + j * m.system_length) * (sy + j * m.system_length);
            int cutoff_x = (int)sqrt((double)(m.position_cutoff_sq - j * j - k * k));
            for (int i = -cutoff_x; i < cutoff_x + 1; i++) {
                double vector_x = sx + i * m.system_length;
                double vector_sq = vector_x * vector_x + vector_y_sq + vector_z_sq;
                double vector_norm = sqrt(vector_sq);
                derivative += vector_x *
                              (m.two_alpha_over_length_root_pi * exp(-m.alpha_over_length_sq * vector_sq) +
                               erfc(m.alpha_over_length * vector_norm) / vector_norm) /
                              vector_sq;
            }
        }
    }
    double delta_cos_x = cos(m.two_pi_over_length * sx);
    double delta_sin_x = sin(m.two_pi_over_length * sx);
    double delta_cos_y = cos(m.two_pi_over_length * sy);
    double delta_sin_y = sin(m.two_pi_over_length * sy);
    double delta_cos_z = cos(m.two_pi_over_length * sz);
    double delta_sin_z = sin(m.two_pi_over_length * sz);
    double cos_x = delta_cos_x, sin_x = delta_sin_x;
    double cos_y = 1.0, sin_y = 0.0, cos_z = 1.0, sin_z = 0.0, store;
    for (int i = 1; i < m.fourier_cutoff + 1; i++) {
        int cutoff_y = (int)sqrt((double)(m.fourier_cutoff_sq - i * i));
        for (int j = 0; j < cutoff_y + 1; j++) {
            int cutoff_x = (int)sqrt((double)(m.fourier_cutoff_sq - i * i - j * j));
            for (int k = 0; k < cutoff_x + 1; k++) {
                derivative += m.fourier[(i * n + j) * n + k] * sin_x * cos_y * cos_z;
                if (k != cutoff_x) {
                    store = cos_z;
                    cos_z = store * delta_cos_z - sin_z * delta_sin_z;
                    sin_z = sin_z * delta_cos_z + store * delta_sin_z;
                } else if (j != cutoff_y) {
                    store = cos_y;
                    cos_y = store * delta_cos_y - sin_y * delta_sin_y;
                    sin_y = sin_y * delta_cos_y + store * delta_sin_y;
                    cos_z = 1.0;
                    sin_z = 0.0;
                } else if (i != m.fourier_cutoff) {
                    store = cos_x;
                    cos_x = store * delta_cos_x - sin_x * delta_sin_x;
                    sin_x = sin_x * delta_cos_x + store * delta_sin_x;
                    cos_y = 1.0;
                    sin_y = 0.0;
                    cos_z = 1.0;
                    sin_z = 0.0;
                }
            }
        }
    }
    return derivative;
}

// MergedImageCoulombPotential.standard_velocity_derivative (.py:128-154)
__device__ inline double mic_std_derivative(const MIC &m, double prefactor, int d, const double *s, double c1, double c2) {
    double p[3];
    permute3(s, d, p);
    return prefactor * c1 * c2 * mic_x(m, p[0], p[1], p[2]);
}

}  // namespace jf
