/*
 * jf_oracle.c -- CPU restatement of JeLLyFysh's event-time path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the GPU product is tested against.  Loaded by tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py; never by the product.
 *
 * Build: gcc -O2 -fPIC -shared -ffp-contract=off (see oracle/build_oracle.py).  The flag
 * keeps every multiply and add a separately rounded IEEE operation, which is what CPython
 * does for Python-level float arithmetic, on x86 and on Arm alike.
 *
 * File map (reference paths relative to the JeLLyFysh source tree):
 *   python float semantics ....... CPython 3.12 float_rem / float_divmod / builtin sum
 *   Time .......................... jellyfysh/base/time.py
 *   vectors ....................... jellyfysh/base/vectors.py
 *   periodic boundaries ........... jellyfysh/setting/hypercubic_setting.py
 *   potentials .................... jellyfysh/potential/ (Python modules and the two C extensions)
 *   cells / occupancy ............. jellyfysh/activator/internal_state/...
 *   estimator / Walker ............ jellyfysh/estimator/inner_point_estimator.py, event_handler/walker.py
 *   event loop .................... jellyfysh/mediator/single_process_mediator.py:91-156 and the
 *                                   event handlers it drives
 */
#include "jf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================================
 * CPython float semantics
 * ==================================================================================== */

/* float.__mod__ (CPython Objects/floatobject.c float_rem): fmod, then the sign of the divisor.
 * Used by HypercubicPeriodicBoundaries.correct_position_entry (hypercubic_setting.py:101-117). */
double jfo_py_mod(double x, double y) {
    double mod = fmod(x, y);
    if (mod != 0.0) {
        if ((y < 0.0) != (mod < 0.0)) mod += y;
    } else {
        mod = copysign(0.0, y);
    }
    return mod;
}

/* divmod(float, float) (CPython float_divmod), used by Time.__add__ / Time.from_float
 * (time.py:87-101, 115-133). */
void jfo_py_divmod(double vx, double wx, double *quotient, double *remainder) {
    double mod = fmod(vx, wx);
    double div = (vx - mod) / wx;
    double floordiv;
    if (mod != 0.0) {
        if ((wx < 0.0) != (mod < 0.0)) {
            mod += wx;
            div -= 1.0;
        }
    } else {
        mod = copysign(0.0, wx);
    }
    if (div != 0.0) {
        floordiv = floor(div);
        if (div - floordiv > 0.5) floordiv += 1.0;
    } else {
        floordiv = copysign(0.0, vx / wx);
    }
    *quotient = floordiv;
    *remainder = mod;
}

/* builtin sum() over floats starting from the int 0 (CPython 3.12 bltinmodule.c): the first
 * item is added to int 0, the rest are accumulated with Neumaier's compensated summation and
 * the compensation is added at the end when it is nonzero and finite. */
double jfo_py_sum(const double *values, int n) {
    if (n == 0) return 0.0;
    double f = 0.0 + values[0];
    double c = 0.0;
    for (int i = 1; i < n; ++i) {
        double x = values[i];
        double t = f + x;
        if (fabs(f) >= fabs(x)) {
            c += (f - t) + x;
        } else {
            c += (x - t) + f;
        }
        f = t;
    }
    if (c != 0.0 && isfinite(c)) f += c;
    return f;
}

double jfo_py_sum3(double a, double b, double c) {
    double v[3] = {a, b, c};
    return jfo_py_sum(v, 3);
}

/* Time.__add__ (time.py:115-133). */
void jfo_time_add(double q, double r, double dt, double *out_q, double *out_r) {
    if (isinf(dt)) {
        *out_q = dt;
        *out_r = dt;
        return;
    }
    double add_q, new_r;
    jfo_py_divmod(r + dt, 1.0, &add_q, &new_r);
    *out_q = q + add_q;
    *out_r = new_r;
}

/* Time.__sub__ (time.py:135-149): self.q - other.q + self.r - other.r, left to right. */
double jfo_time_sub(double q1, double r1, double q2, double r2) {
    return ((q1 - q2) + r1) - r2;
}

/* Time.__lt__ (time.py:167-182). */
int jfo_time_lt(double q1, double r1, double q2, double r2) {
    return q1 < q2 || (q1 == q2 && r1 < r2);
}

/* ======================================================================================
 * Keyed random numbers.
 *
 * The reference draws from Python's global Mersenne Twister in an order that depends on
 * set iteration over Cell objects hashed by address, so a shared seed cannot reproduce its
 * draws.  Parity runs instead key every draw by (chain, event index, kind, target) through
 * the SplitMix64 output function (Steele, Lea and Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014) applied to a Weyl-sequence state; the reference is driven with
 * the same numbers by replacing its random-module calls.
 * ==================================================================================== */
static uint64_t jfo_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

#define JFO_GOLDEN 0x9e3779b97f4a7c15ULL

uint64_t jfo_chain_key(uint64_t seed, uint64_t chain) {
    return jfo_mix64(seed + (chain + 1) * JFO_GOLDEN);
}

uint64_t jfo_draw(uint64_t key, uint64_t event, uint32_t kind, uint32_t target) {
    uint64_t counter = (event << 24) | ((uint64_t)(kind & 0xF) << 20) | (uint64_t)(target & 0xFFFFF);
    return jfo_mix64(key + (counter + 1) * JFO_GOLDEN);
}

/* 53-bit uniform in [0, 1), the same lattice as random.random(). */
double jfo_uniform(uint64_t bits) {
    return (double)(bits >> 11) * (1.0 / 9007199254740992.0);
}

/* Natural logarithm for x in (0, inf), written out so that the CPU and the GPU produce the same
 * bits: x = 2^e m with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(f), f = (m - 1)/(m + 1),
 * atanh by its Taylor series (Abramowitz & Stegun 4.1.27) to f^23, log 2 split in a head
 * with trailing zeros and a tail.  Accuracy is about one ulp. */
double jfo_log(double x) {
    uint64_t bits;
    memcpy(&bits, &x, sizeof(bits));
    int e = (int)((bits >> 52) & 0x7FF);
    if (e == 0) { /* subnormal: scale into the normal range */
        x = x * 18014398509481984.0; /* 2^54 */
        memcpy(&bits, &x, sizeof(bits));
        e = (int)((bits >> 52) & 0x7FF) - 54;
    }
    e -= 1023;
    uint64_t mbits = (bits & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL;
    double m;
    memcpy(&m, &mbits, sizeof(m));
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
    const double ln2_hi = 6.93147180369123816490e-01; /* 0x3fe62e42fee00000 */
    const double ln2_lo = 1.90821492927058770002e-10; /* 0x3dea39ef35793c76 */
    return de * ln2_hi + (de * ln2_lo + log_m);
}

/* random.expovariate(beta) = -log(1.0 - random()) / beta. */
double jfo_expovariate(uint64_t bits, double beta) {
    return -jfo_log(1.0 - jfo_uniform(bits)) / beta;
}

/* integer in [0, n) from the high 32 bits (multiply-shift). */
uint32_t jfo_randbelow(uint64_t bits, uint32_t n) {
    return (uint32_t)(((bits >> 32) * (uint64_t)n) >> 32);
}

/* ======================================================================================
 * vectors (jellyfysh/base/vectors.py)
 * ==================================================================================== */
static double norm_sq3(const double *v) { /* vectors.norm_sq :   sum(c * c) */
    return jfo_py_sum3(v[0] * v[0], v[1] * v[1], v[2] * v[2]);
}

static double norm3(const double *v) { /* vectors.norm : sum(c * c) ** 0.5 */
    return pow(norm_sq3(v), 0.5);
}

/* sum([value ** 2 for index, value in enumerate(v) if index != d]) (vectors.py:181, 213);
 * a two-term Neumaier sum equals the plain sum. */
static double perp_sq(const double *v, int d) {
    double a[2];
    int k = 0;
    for (int i = 0; i < 3; ++i)
        if (i != d) a[k++] = pow(v[i], 2.0);
    return jfo_py_sum(a, 2);
}

/* vectors.displacement_until_new_norm_sq_component_positive (vectors.py:153-181) */
static int disp_until_positive(const double *v, double norm_sq_new, int d, double *out) {
    if (!(v[d] > 0.0)) return JFO_ASSERT;
    double radicand = norm_sq_new - perp_sq(v, d);
    if (radicand < 0.0) return JFO_VALUE_ERROR;
    *out = v[d] - sqrt(radicand);
    return JFO_OK;
}

/* vectors.displacement_until_new_norm_sq_component_negative (vectors.py:184-214) */
static int disp_until_negative(const double *v, double norm_sq_new, int d, double *out) {
    if (!(v[d] <= 0.0)) return JFO_ASSERT;
    double radicand = norm_sq_new - perp_sq(v, d);
    if (radicand < 0.0) return JFO_VALUE_ERROR;
    *out = v[d] + sqrt(radicand);
    return JFO_OK;
}

/* StandardVelocityPotential._analyse_velocity (potential/abstracts.py:115-140) */
static int analyse_velocity(const double *velocity, int *direction, double *speed) {
    int count = 0, dir = -1;
    for (int i = 0; i < 3; ++i)
        if (velocity[i] != 0.0) {
            ++count;
            dir = i;
        }
    if (count != 1 || !(velocity[dir] > 0.0)) return JFO_ASSERT;
    *direction = dir;
    *speed = velocity[dir];
    return JFO_OK;
}

/* Python float division: raises ZeroDivisionError for a zero divisor. */
#define PYDIV(a, b, out)                                                                          \
    do {                                                                                          \
        double divisor_ = (b);                                                                    \
        if (divisor_ == 0.0) return JFO_ZERO_DIVISION;                                            \
        (out) = (a) / divisor_;                                                                   \
    } while (0)

/* Python float ** float: negative base with a fractional exponent gives a complex number. */
static int py_pow(double x, double y, double *out) {
    if (x < 0.0 && y != floor(y)) return JFO_COMPLEX;
    if (x == 0.0 && y < 0.0) return JFO_ZERO_DIVISION;
    *out = pow(x, y);
    return JFO_OK;
}

/* ======================================================================================
 * Hard sphere (potential/hard_sphere_potential.py:65-99)
 * ==================================================================================== */
int jfo_hs_displacement(double radius, const double *velocity, const double *separation, double *out) {
    double diameter_squared = 4.0 * radius * radius;
    double velocity_squared = norm_sq3(velocity);
    if (!(velocity_squared > 0.0)) return JFO_ASSERT;
    double separation_squared = norm_sq3(separation);
    if (!(separation_squared - diameter_squared > -1.0e-13)) return JFO_ASSERT;
    double vds = jfo_py_sum3(velocity[0] * separation[0], velocity[1] * separation[1],
                             velocity[2] * separation[2]);
    double square_root_term = vds * vds - velocity_squared * (separation_squared - diameter_squared);
    if (square_root_term >= 0.0 && vds >= 0.0) {
        *out = (vds - sqrt(square_root_term)) / velocity_squared;
    } else {
        *out = INFINITY;
    }
    return JFO_OK;
}

/* ======================================================================================
 * Inverse power potential (potential/inverse_power_potential.py)
 * ==================================================================================== */
typedef struct {
    double power, prefactor, two_over_power, power_over_two, power_plus_two;
} IP;

static IP ip_make(double power, double prefactor) {
    IP p;
    p.power = power;
    p.prefactor = prefactor;
    p.two_over_power = 2.0 / power;
    p.power_over_two = power / 2.0;
    p.power_plus_two = power + 2.0;
    return p;
}

/* InversePowerPotential.potential (:127-143): charge_product * k / norm_sq ** (p / 2) */
static int ip_potential(const IP *p, double charge_product, const double *s, double *out) {
    double denominator;
    int st = py_pow(norm_sq3(s), p->power_over_two, &denominator);
    if (st) return st;
    PYDIV(charge_product * p->prefactor, denominator, *out);
    return JFO_OK;
}

/* InversePowerPotential.standard_velocity_derivative (:71-94) */
static int ip_std_derivative(const IP *p, int d, const double *s, double c1, double c2, double *out) {
    double denominator;
    int st = py_pow(norm3(s), p->power_plus_two, &denominator);
    if (st) return st;
    double value;
    PYDIV(p->power * s[d], denominator, value);
    *out = ((value * p->prefactor) * c1) * c2;
    return JFO_OK;
}

/* InversePowerPotential._displacement_repulsive (:145-161) */
static int ip_repulsive(const IP *p, int d, double cp, double du, double *s, double *out) {
    if (s[d] <= 0.0) {
        *out = INFINITY;
        return JFO_OK;
    }
    double s_max[3] = {s[0], s[1], s[2]};
    s_max[d] = 0.0;
    double maximum_potential, current_potential;
    int st = ip_potential(p, cp, s_max, &maximum_potential);
    if (st) return st;
    st = ip_potential(p, cp, s, &current_potential);
    if (st) return st;
    if (du < maximum_potential - current_potential) {
        double ratio, nsq;
        PYDIV(cp * p->prefactor, current_potential + du, ratio);
        st = py_pow(ratio, p->two_over_power, &nsq);
        if (st) return st;
        return disp_until_positive(s, nsq, d, out);
    }
    *out = INFINITY;
    return JFO_OK;
}

/* InversePowerPotential._displacement_attractive (:163-179) */
static int ip_attractive(const IP *p, int d, double cp, double du, double *s, double *out) {
    double displacement = 0.0;
    if (s[d] > 0.0) {
        displacement += s[d];
        s[d] = 0.0;
    }
    double current_potential;
    int st = ip_potential(p, cp, s, &current_potential);
    if (st) return st;
    if (current_potential + du >= 0.0) {
        *out = INFINITY;
        return JFO_OK;
    }
    double ratio, nsq, extra;
    PYDIV(cp * p->prefactor, current_potential + du, ratio);
    st = py_pow(ratio, p->two_over_power, &nsq);
    if (st) return st;
    st = disp_until_negative(s, nsq, d, &extra);
    if (st) return st;
    *out = displacement + extra;
    return JFO_OK;
}

int jfo_ip_displacement(double power, double prefactor, const double *velocity, const double *separation,
                        double charge_one, double charge_two, double potential_change, double *out) {
    int d;
    double speed;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    IP p = ip_make(power, prefactor);
    double s[3] = {separation[0], separation[1], separation[2]};
    double cp = charge_one * charge_two;
    double disp;
    st = (p.prefactor * cp > 0.0) ? ip_repulsive(&p, d, cp, potential_change, s, &disp)
                                  : ip_attractive(&p, d, cp, potential_change, s, &disp);
    if (st) return st;
    *out = disp / speed;
    return JFO_OK;
}

int jfo_ip_derivative(double power, double prefactor, const double *velocity, const double *separation,
                      double charge_one, double charge_two, double *out) {
    int d;
    double speed, value;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    IP p = ip_make(power, prefactor);
    st = ip_std_derivative(&p, d, separation, charge_one, charge_two, &value);
    if (st) return st;
    *out = value * speed;
    return JFO_OK;
}

/* ======================================================================================
 * Mexican-hat potentials (potential/abstracts.py:336-530) with the Lennard-Jones
 * (potential/lennard_jones_potential.py) and displaced-even-power
 * (potential/displaced_even_power_potential.py) specialisations.
 * ==================================================================================== */
typedef struct {
    int kind; /* 0 Lennard-Jones, 1 displaced even power */
    double prefactor;
    double r0, r0_squared;
    /* Lennard-Jones */
    double sigma;
    IP six, twelve;
    /* displaced even power */
    double power, inverse_power;
} MH;

static MH mh_lj(double prefactor, double sigma) {
    MH h;
    memset(&h, 0, sizeof(h));
    h.kind = 0;
    h.prefactor = prefactor;
    h.sigma = sigma;
    h.r0 = sigma * pow(2.0, 1.0 / 6.0);        /* characteristic_length * 2 ** (1 / 6) */
    h.r0_squared = pow(h.r0, 2.0);              /* equilibrium_separation ** 2 */
    h.six = ip_make(6.0, -prefactor * pow(sigma, 6.0));
    h.twelve = ip_make(12.0, prefactor * pow(sigma, 12.0));
    return h;
}

static MH mh_dep(double r0, int power, double prefactor) {
    MH h;
    memset(&h, 0, sizeof(h));
    h.kind = 1;
    h.prefactor = prefactor;
    h.r0 = r0;
    h.r0_squared = pow(r0, 2.0);
    h.power = (double)power;
    h.inverse_power = 1.0 / (double)power;
    return h;
}

static int mh_potential(const MH *h, const double *s, double *out) {
    if (h->kind == 0) { /* lennard_jones_potential.py:83-98 */
        double a, b;
        int st = ip_potential(&h->six, 1.0, s, &a);
        if (st) return st;
        st = ip_potential(&h->twelve, 1.0, s, &b);
        if (st) return st;
        *out = a + b;
        return JFO_OK;
    }
    /* displaced_even_power_potential.py:95-110 */
    double distance = norm3(s) - h->r0;
    double powered;
    int st = py_pow(distance, h->power, &powered);
    if (st) return st;
    *out = h->prefactor * powered;
    return JFO_OK;
}

static int mh_invert_inside(const MH *h, double potential, double *out) {
    if (h->kind == 0) { /* lennard_jones_potential.py:100-115 */
        double root, sigma_over_r_six, denominator;
        int st = py_pow(1.0 + (4.0 * potential) / h->prefactor, 0.5, &root);
        if (st) return st;
        sigma_over_r_six = (1.0 + root) / 2.0;
        st = py_pow(sigma_over_r_six, 1.0 / 6.0, &denominator);
        if (st) return st;
        PYDIV(h->sigma, denominator, *out);
        return JFO_OK;
    }
    double powered; /* displaced_even_power_potential.py:112-126 */
    int st = py_pow(potential / h->prefactor, h->inverse_power, &powered);
    if (st) return st;
    *out = h->r0 - powered;
    return JFO_OK;
}

static int mh_invert_outside(const MH *h, double potential, double *out) {
    if (h->kind == 0) { /* lennard_jones_potential.py:117-135 */
        if (potential >= 0.0) {
            *out = INFINITY;
            return JFO_OK;
        }
        double root, denominator;
        int st = py_pow(1.0 + (4.0 * potential) / h->prefactor, 0.5, &root);
        if (st) return st;
        double sigma_over_r_six = (1.0 - root) / 2.0;
        st = py_pow(sigma_over_r_six, 1.0 / 6.0, &denominator);
        if (st) return st;
        PYDIV(h->sigma, denominator, *out);
        return JFO_OK;
    }
    double powered; /* displaced_even_power_potential.py:128-142 */
    int st = py_pow(potential / h->prefactor, h->inverse_power, &powered);
    if (st) return st;
    *out = h->r0 + powered;
    return JFO_OK;
}

static int mh_front_inside(const MH *h, int d, double du, double *s, double *out);

/* _displacement_front_outside_sphere (abstracts.py:384-408) */
static int mh_front_outside(const MH *h, int d, double u, double du, double *s, double *out) {
    double norm_new;
    int st = mh_invert_outside(h, u + du, &norm_new);
    if (st) return st;
    return disp_until_negative(s, norm_new * norm_new, d, out);
}

/* _displacement_behind_inside_sphere (abstracts.py:486-530) */
static int mh_behind_inside(const MH *h, int d, double u, double du, double *s, double *out) {
    double s_max[3] = {s[0], s[1], s[2]};
    s_max[d] = 0.0;
    double u_max;
    int st = mh_potential(h, s_max, &u_max);
    if (st) return st;
    double difference = u_max - u;
    if (du < difference) {
        double norm_new;
        st = mh_invert_inside(h, u + du, &norm_new);
        if (st) return st;
        return disp_until_positive(s, norm_new * norm_new, d, out);
    }
    double displacement = s[d];
    s[d] = 0.0;
    du -= difference;
    double extra;
    st = mh_front_inside(h, d, du, s, &extra);
    if (st) return st;
    *out = displacement + extra;
    return JFO_OK;
}

/* _displacement_front_inside_sphere (abstracts.py:456-484) */
static int mh_front_inside(const MH *h, int d, double du, double *s, double *out) {
    double displacement, u, extra;
    int st = disp_until_negative(s, h->r0_squared, d, &displacement);
    if (st) return st;
    s[d] -= displacement;
    st = mh_potential(h, s, &u);
    if (st) return st;
    st = mh_front_outside(h, d, u, du, s, &extra);
    if (st) return st;
    *out = displacement + extra;
    return JFO_OK;
}

/* _displacement_behind_outside_sphere (abstracts.py:410-454): a ValueError anywhere in the try
 * block switches to the fallback, which sees the separation as mutated up to that point. */
static int mh_behind_outside(const MH *h, int d, double du, double *s, double *out) {
    double displacement, u, extra;
    int st = disp_until_positive(s, h->r0_squared, d, &displacement);
    if (st == JFO_OK) {
        s[d] -= displacement;
        st = mh_potential(h, s, &u);
        if (st == JFO_OK) {
            st = mh_behind_inside(h, d, u, du, s, &extra);
            if (st == JFO_OK) {
                *out = displacement + extra;
                return JFO_OK;
            }
        }
    }
    if (st != JFO_VALUE_ERROR) return st;
    displacement = s[d];
    s[d] = 0.0;
    st = mh_potential(h, s, &u);
    if (st) return st;
    st = mh_front_outside(h, d, u, du, s, &extra);
    if (st) return st;
    *out = displacement + extra;
    return JFO_OK;
}

/* MexicanHatPotential.standard_velocity_displacement (abstracts.py:336-382) */
static int mh_std_displacement(const MH *h, int d, double *s, double du, double *out) {
    double norm = norm3(s);
    if (norm >= h->r0) {
        if (s[d] <= 0.0) {
            double u;
            int st = mh_potential(h, s, &u);
            if (st) return st;
            return mh_front_outside(h, d, u, du, s, out);
        }
        return mh_behind_outside(h, d, du, s, out);
    }
    if (s[d] <= 0.0) return mh_front_inside(h, d, du, s, out);
    double u;
    int st = mh_potential(h, s, &u);
    if (st) return st;
    return mh_behind_inside(h, d, u, du, s, out);
}

static int mh_std_derivative(const MH *h, int d, const double *s, double *out) {
    if (h->kind == 0) { /* lennard_jones_potential.py:63-81 */
        double a, b;
        int st = ip_std_derivative(&h->six, d, s, 1.0, 1.0, &a);
        if (st) return st;
        st = ip_std_derivative(&h->twelve, d, s, 1.0, 1.0, &b);
        if (st) return st;
        *out = a + b;
        return JFO_OK;
    }
    /* displaced_even_power_potential.py:73-93 */
    double norm = norm3(s);
    double powered;
    int st = py_pow(norm - h->r0, h->power - 1.0, &powered);
    if (st) return st;
    PYDIV((((-h->power) * h->prefactor) * powered) * s[d], norm, *out);
    return JFO_OK;
}

static int mh_displacement(const MH *h, const double *velocity, const double *separation, double du,
                           double *out) {
    int d;
    double speed, disp;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    double s[3] = {separation[0], separation[1], separation[2]};
    st = mh_std_displacement(h, d, s, du, &disp);
    if (st) return st;
    *out = disp / speed;
    return JFO_OK;
}

static int mh_derivative(const MH *h, const double *velocity, const double *separation, double *out) {
    int d;
    double speed, value;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    st = mh_std_derivative(h, d, separation, &value);
    if (st) return st;
    *out = value * speed;
    return JFO_OK;
}

int jfo_lj_displacement(double prefactor, double sigma, const double *velocity, const double *separation,
                        double potential_change, double *out) {
    MH h = mh_lj(prefactor, sigma);
    return mh_displacement(&h, velocity, separation, potential_change, out);
}

int jfo_lj_derivative(double prefactor, double sigma, const double *velocity, const double *separation,
                      double *out) {
    MH h = mh_lj(prefactor, sigma);
    return mh_derivative(&h, velocity, separation, out);
}

int jfo_dep_displacement(double r0, int power, double prefactor, const double *velocity,
                         const double *separation, double potential_change, double *out) {
    MH h = mh_dep(r0, power, prefactor);
    return mh_displacement(&h, velocity, separation, potential_change, out);
}

int jfo_dep_derivative(double r0, int power, double prefactor, const double *velocity,
                       const double *separation, double *out) {
    MH h = mh_dep(r0, power, prefactor);
    return mh_derivative(&h, velocity, separation, out);
}

/* ======================================================================================
 * Inverse-power Coulomb bounding potential
 * (potential/inverse_power_coulomb_bounding_potential/inverse_power_coulomb_bounding_potential.c:53-139
 *  and .py:111-140; the Python wrapper permutes the separation so that x is the motion axis,
 *  base/vectors.py:220-239)
 * ==================================================================================== */
static void permute3(const double *s, int d, double *p) {
    p[0] = s[d];
    p[1] = s[(d + 1) % 3];
    p[2] = s[(d + 2) % 3];
}

static double ipcb_x_derivative(double pp, double sx, double sy, double sz) {
    return pp * sx / pow(sx * sx + sy * sy + sz * sz, 3.0 / 2.0);
}

static double ipcb_potential(double pp, double sx, double sy, double sz) {
    return pp / sqrt(sx * sx + sy * sy + sz * sz);
}

static double ipcb_x_displacement(double pp, double sx, double sy, double sz, double du, double length) {
    double half = length / 2.0;
    double current = ipcb_potential(pp, sx, sy, sz);
    double u_zero = ipcb_potential(pp, 0.0, sy, sz);
    double u_half = ipcb_potential(pp, half, sy, sz);
    double per_length = fabs(u_zero - u_half);
    double displacement = floor(du / per_length) * length;
    du = fmod(du, per_length);
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

int jfo_ipcb_displacement(double prefactor, double system_length, const double *velocity,
                          const double *separation, double charge_one, double charge_two,
                          double potential_change, double *out) {
    int d;
    double speed, p[3];
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    permute3(separation, d, p);
    double disp = ipcb_x_displacement(prefactor * charge_one * charge_two, p[0], p[1], p[2], potential_change,
                                      system_length);
    *out = disp / speed;
    return JFO_OK;
}

int jfo_ipcb_derivative(double prefactor, const double *velocity, const double *separation, double charge_one,
                        double charge_two, double *out) {
    int d;
    double speed, p[3];
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    permute3(separation, d, p);
    *out = ipcb_x_derivative(prefactor * charge_one * charge_two, p[0], p[1], p[2]) * speed;
    return JFO_OK;
}

/* ======================================================================================
 * Merged-image Coulomb potential
 * (potential/merged_image_coulomb_potential/merged_image_coulomb_potential.c:77-274, .py:128-154)
 * ==================================================================================== */
typedef struct {
    int fourier_cutoff, fourier_cutoff_sq, position_cutoff, position_cutoff_sq;
    double alpha_over_length, alpha_over_length_sq, two_alpha_over_length_root_pi, system_length,
        two_pi_over_length;
    double *fourier; /* [(fc+1)^3], index (i*(fc+1)+j)*(fc+1)+k */
} MIC;

static int mic_init(MIC *m, int fourier_cutoff, int position_cutoff, double alpha, double system_length) {
    int n = fourier_cutoff + 1;
    m->fourier = (double *)calloc((size_t)n * n * n, sizeof(double));
    if (!m->fourier) return JFO_ALLOC;
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++)
            for (int i = 1; i < n; i++) {
                double coefficient;
                if (j == 0 && k == 0)
                    coefficient = 1.0;
                else if (k == 0 || j == 0)
                    coefficient = 2.0;
                else
                    coefficient = 4.0;
                double norm_sq = i * i + j * j + k * k;
                m->fourier[(i * n + j) * n + k] = 4.0 * i * coefficient / (norm_sq * system_length * system_length) *
                                                  exp(-M_PI * M_PI * norm_sq / (alpha * alpha));
            }
    m->fourier_cutoff = fourier_cutoff;
    m->fourier_cutoff_sq = fourier_cutoff * fourier_cutoff;
    m->position_cutoff = position_cutoff;
    m->position_cutoff_sq = position_cutoff * position_cutoff;
    m->alpha_over_length = alpha / system_length;
    m->alpha_over_length_sq = alpha * alpha / (system_length * system_length);
    m->two_alpha_over_length_root_pi = 2.0 * alpha / (system_length * sqrt(M_PI));
    m->system_length = system_length;
    m->two_pi_over_length = 2.0 * M_PI / system_length;
    return JFO_OK;
}

static double mic_x(const MIC *m, double sx, double sy, double sz) {
    double derivative = 0.0;
    int n = m->fourier_cutoff + 1;
    for (int k = -m->position_cutoff; k < m->position_cutoff + 1; k++) {
        double vector_z_sq = (sz + k * m->system_length) * (sz + k * m->system_length);
        int cutoff_y = (int)sqrt(m->position_cutoff_sq - k * k);
        for (int j = -cutoff_y; j < cutoff_y + 1; j++) {
            double vector_y_sq = (sy + j * m->system_length) * (sy + j * m->system_length);
            int cutoff_x = (int)sqrt(m->position_cutoff_sq - j * j - k * k);
            for (int i = -cutoff_x; i < cutoff_x + 1; i++) {
                double vector_x = sx + i * m->system_length;
                double vector_sq = vector_x * vector_x + vector_y_sq + vector_z_sq;
                double vector_norm = sqrt(vector_sq);
                derivative += vector_x *
                              (m->two_alpha_over_length_root_pi * exp(-m->alpha_over_length_sq * vector_sq) +
                               erfc(m->alpha_over_length * vector_norm) / vector_norm) /
                              vector_sq;
            }
        }
    }
    double delta_cos_x = cos(m->two_pi_over_length * sx);
    double delta_sin_x = sin(m->two_pi_over_length * sx);
    double delta_cos_y = cos(m->two_pi_over_length * sy);
    double delta_sin_y = sin(m->two_pi_over_length * sy);
    double delta_cos_z = cos(m->two_pi_over_length * sz);
    double delta_sin_z = sin(m->two_pi_over_length * sz);
    double cos_x = delta_cos_x, sin_x = delta_sin_x;
    double cos_y = 1.0, sin_y = 0.0, cos_z = 1.0, sin_z = 0.0, store;
    for (int i = 1; i < m->fourier_cutoff + 1; i++) {
        int cutoff_y = (int)sqrt(m->fourier_cutoff_sq - i * i);
        for (int j = 0; j < cutoff_y + 1; j++) {
            int cutoff_x = (int)sqrt(m->fourier_cutoff_sq - i * i - j * j);
            for (int k = 0; k < cutoff_x + 1; k++) {
                derivative += m->fourier[(i * n + j) * n + k] * sin_x * cos_y * cos_z;
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
                } else if (i != m->fourier_cutoff) {
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

double jfo_mic_x_derivative(double alpha, int fourier_cutoff, int position_cutoff, double system_length,
                            double sx, double sy, double sz) {
    MIC m;
    if (mic_init(&m, fourier_cutoff, position_cutoff, alpha, system_length)) return NAN;
    double value = mic_x(&m, sx, sy, sz);
    free(m.fourier);
    return value;
}

static double mic_std_derivative(const MIC *m, double prefactor, int d, const double *s, double c1, double c2) {
    double p[3];
    permute3(s, d, p);
    return prefactor * c1 * c2 * mic_x(m, p[0], p[1], p[2]);
}

int jfo_mic_derivative(double alpha, int fourier_cutoff, int position_cutoff, double prefactor,
                       double system_length, const double *velocity, const double *separation,
                       double charge_one, double charge_two, double *out) {
    int d;
    double speed;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    MIC m;
    if (mic_init(&m, fourier_cutoff, position_cutoff, alpha, system_length)) return JFO_ALLOC;
    *out = mic_std_derivative(&m, prefactor, d, separation, charge_one, charge_two) * speed;
    free(m.fourier);
    return JFO_OK;
}

/* ======================================================================================
 * Composite objects (event_handler/two_composite_object_summed_bounding_potential_event_handler.py)
 * ==================================================================================== */

/* setting.periodic_boundaries.separation_vector (hypercubic_setting.py:120-140, :156-172) */
static void composite_separation(double length, const double *from, const double *to, double *s) {
    double half = length / 2.0;
    for (int d = 0; d < 3; ++d) s[d] = jfo_py_mod((to[d] - from[d]) + half, length) - half;
}

/* send_event_time (:119-150): min() over the target units of the bounding displacement */
int jfo_composite_event_time(int units, double alpha, int fourier_cutoff, int position_cutoff,
                             double coulomb_prefactor, double bound_prefactor, double system_length,
                             const double *velocity, const double *active_position, double active_charge,
                             const double *target_positions, const double *target_charges,
                             const double *potential_changes, double *displacement) {
    (void)alpha;
    (void)fourier_cutoff;
    (void)position_cutoff;
    (void)coulomb_prefactor;
    for (int j = 0; j < units; ++j) {
        double s[3], value;
        composite_separation(system_length, active_position, target_positions + 3 * j, s);
        int st = jfo_ipcb_displacement(bound_prefactor, system_length, velocity, s, active_charge,
                                       target_charges[j], potential_changes[j], &value);
        if (st) return st;
        if (j == 0 || value < *displacement) *displacement = value;
    }
    return JFO_OK;
}

/* send_out_state (:152-202) with _fill_lifting (event_handler_with_bounding_potential.py:170-220).  given: NULL for
 * the summed inverse-power bound of this handler, else the bounding event rate the thinning draws against (the
 * molecular cell-bounding and cell-veto handlers). */
static int composite_out_state(int units, int scheme, int unit_draw, double alpha, int fourier_cutoff,
                               int position_cutoff, double coulomb_prefactor, double bound_prefactor,
                               double system_length, const double *velocity, const double *local_positions,
                               const double *local_charges, int active_index, const double *target_positions,
                               const double *target_charges, int local_first, const double *given,
                               const double *draws, int *new_active, double *bounding_rate, double *event_rate) {
    const double *active = local_positions + 3 * active_index;
    double active_charge = local_charges[active_index];
    double *target_factor = (double *)calloc((size_t)units, sizeof(double));
    double *local_factor = (double *)calloc((size_t)units, sizeof(double));
    double *table = (double *)malloc(sizeof(double) * (size_t)(2 * units));
    int32_t *flags = (int32_t *)malloc(sizeof(int32_t) * (size_t)(2 * units));
    int st = JFO_OK;
    double bounding = 0.0, factor = 0.0;
    *new_active = -1;
    for (int j = 0; j < units && !st; ++j) {
        double s[3], b, pair;
        composite_separation(system_length, active, target_positions + 3 * j, s);
        b = 0.0;
        if (!given) st = jfo_ipcb_derivative(bound_prefactor, velocity, s, active_charge, target_charges[j], &b);
        if (!st) st = jfo_mic_derivative(alpha, fourier_cutoff, position_cutoff, coulomb_prefactor, system_length,
                                         velocity, s, active_charge, target_charges[j], &pair);
        if (st) break;
        bounding += b > 0.0 ? b : 0.0;  /* max(0.0, b) keeps 0.0 unless b is larger */
        factor += pair;
        target_factor[j] -= pair;
    }
    double rate = factor > 0.0 ? factor : 0.0;
    if (given) {
        bounding = *given;
        /* assert bounding_event_rate >= 0.0 (two_composite_object_cell_bounding_potential_event_handler.py:243,
         * composite_object_cell_veto_event_handler.py:150) */
        if (!st && !(bounding >= 0.0)) st = JFO_ASSERT;
    }
    *bounding_rate = bounding;
    *event_rate = rate;
    double thinning = unit_draw ? 0.0 + (bounding - 0.0) * draws[0] : draws[0];
    if (!st && !(rate <= thinning)) {
        for (int i = 0; i < units && !st; ++i) {
            if (i == active_index) {
                local_factor[i] = rate;
                continue;
            }
            for (int j = 0; j < units; ++j) {
                double s[3], pair;
                composite_separation(system_length, local_positions + 3 * i, target_positions + 3 * j, s);
                st = jfo_mic_derivative(alpha, fourier_cutoff, position_cutoff, coulomb_prefactor, system_length,
                                        velocity, s, local_charges[i], target_charges[j], &pair);
                if (st) break;
                local_factor[i] += pair;
                target_factor[j] -= pair;
            }
        }
        if (!st) {
            /* insertion order of the derivative table: the object with the smaller identifier first */
            int n = 0;
            for (int pass = 0; pass < 2; ++pass) {
                int locals = (pass == 0) == (local_first != 0);
                for (int i = 0; i < units; ++i, ++n) {
                    table[n] = locals ? local_factor[i] : target_factor[i];
                    flags[n] = locals && i == active_index;
                }
            }
            int64_t selected;
            double bound;
            st = jfo_lifting(scheme, unit_draw, table, flags, 2 * units, scheme == 2 ? draws[2] : draws[1],
                             &selected, &bound);
            if (!st) {
                int local_start = local_first ? 0 : units;
                int index = (int)selected;
                *new_active = (index >= local_start && index < local_start + units) ? index - local_start
                                                                                    : units + (index - (units - local_start));
            }
        }
    }
    free(target_factor);
    free(local_factor);
    free(table);
    free(flags);
    return st;
}

int jfo_composite_out_state(int units, int scheme, int unit_draw, double alpha, int fourier_cutoff,
                            int position_cutoff, double coulomb_prefactor, double bound_prefactor,
                            double system_length, const double *velocity, const double *local_positions,
                            const double *local_charges, int active_index, const double *target_positions,
                            const double *target_charges, int local_first, const double *draws, int *new_active,
                            double *bounding_rate, double *event_rate) {
    return composite_out_state(units, scheme, unit_draw, alpha, fourier_cutoff, position_cutoff, coulomb_prefactor,
                               bound_prefactor, system_length, velocity, local_positions, local_charges,
                               active_index, target_positions, target_charges, local_first, NULL, draws, new_active,
                               bounding_rate, event_rate);
}

/* send_out_state of the molecular cell-bounding handler
 * (two_composite_object_cell_bounding_potential_event_handler.py:231-265) and of the molecular cell veto with a
 * target (composite_object_cell_veto_event_handler.py:131-162): the summed merged-image derivative of the active
 * unit against the target object, thinned against the given bounding event rate, then _fill_lifting and the
 * lifting scheme. */
int jfo_composite_bounded_out_state(int units, int scheme, int unit_draw, double alpha, int fourier_cutoff,
                                    int position_cutoff, double coulomb_prefactor, double system_length,
                                    const double *velocity, const double *local_positions,
                                    const double *local_charges, int active_index, const double *target_positions,
                                    const double *target_charges, int local_first, double bounding_rate,
                                    const double *draws, int *new_active, double *event_rate) {
    double bounding;
    return composite_out_state(units, scheme, unit_draw, alpha, fourier_cutoff, position_cutoff, coulomb_prefactor,
                               0.0, system_length, velocity, local_positions, local_charges, active_index,
                               target_positions, target_charges, local_first, &bounding_rate, draws, new_active,
                               &bounding, event_rate);
}

/* CellBoundingPotential.standard_velocity_displacement (cell_bounding_potential.py:155-198) through
 * Potential.displacement (potential/abstracts.py:212-245), with the charge factor of
 * DipoleMonteCarloEstimator.charge_correction_factor (estimator/dipole_monte_carlo_estimator.py:157-190): the active
 * charge times the largest absolute target charge over the estimator's dipole charge (the target charges summing to
 * 0.0 by the builtin sum).  upper / lower are the bounds of the relative cell in the three directions; rate is the
 * stored bounding event rate (per unit length: the out-state draws against rate times the speed), time the time
 * displacement. */
int jfo_composite_cell_bound_time(const double *upper, const double *lower, const double *velocity,
                                  double active_charge,
                                  const double *target_charges, int units, double dipole_charge,
                                  double potential_change, double *rate, double *time) {
    int d;
    double speed;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    if (units < 1 || jfo_py_sum(target_charges, units) != 0.0) return JFO_ASSERT;
    if (isnan(upper[d]) || isnan(lower[d])) return JFO_ASSERT;  /* a nearby relative cell: no bound */
    double largest = fabs(target_charges[0]);
    for (int j = 1; j < units; ++j)
        if (fabs(target_charges[j]) > largest) largest = fabs(target_charges[j]);
    if (dipole_charge == 0.0) return JFO_ZERO_DIVISION;
    double product = active_charge * largest / dipole_charge;
    *rate = product > 0.0 ? upper[d] * product : lower[d] * product;
    double displacement = *rate > 0 ? potential_change / *rate : INFINITY;
    *time = displacement / speed;
    return JFO_OK;
}

/* CellVetoEventHandler.send_event_time (abstracts/cell_veto_event_handler.py:200-238) for a composite object, whose
 * charge factor is the active charge (DipoleMonteCarloEstimator.charge_correction_factor without target charges):
 * positive, the upper bounds and their Walker table's total rate (walker_upper, one per direction); else its
 * negative, the lower ones.  upper / lower are the bounds of the sampled relative cell in the three directions; rate
 * is the bounding event rate of the out-state, time the time displacement potential_change / (total rate * speed). */
int jfo_composite_cell_veto_time(const double *upper, const double *lower, const double *walker_upper,
                                 const double *walker_lower, const double *velocity, double active_charge,
                                 double potential_change, double *rate, double *time) {
    int d;
    double speed;
    int st = analyse_velocity(velocity, &d, &speed);
    if (st) return st;
    double factor = active_charge, total, bound;
    if (factor > 0.0) {
        total = walker_upper[d];
        bound = upper[d];
    } else {
        factor *= -1.0;
        total = walker_lower[d];
        bound = lower[d];
    }
    double total_rate = total * factor;
    *rate = bound * factor;
    if (!(*rate > 0.0)) return JFO_ASSERT;
    double denominator = total_rate * speed;
    if (denominator == 0.0) return JFO_ZERO_DIVISION;
    *time = potential_change / denominator;
    return JFO_OK;
}

/* ======================================================================================
 * Cells (activator/internal_state/cell_occupancy/cells/cuboid_cells.py,
 *        cuboid_periodic_cells.py)
 * ==================================================================================== */
static double next_up(double x) {
    if (isnan(x) || (isinf(x) && x > 0)) return x;
    if (x == 0.0) x = 0.0;
    return nextafter(x, INFINITY);
}

static double next_down(double x) { return -next_up(-x); }

/* exact float bounds of the cells along one axis (cuboid_cells.py:115-131) */
/* ---- lifting schemes ---------------------------------------------------------------------------------- */

/* random.uniform(a, b) = a + (b - a) * random() (Python 3.12 random.py) */
static double py_uniform(double a, double b, double unit) { return a + (b - a) * unit; }

int jfo_lifting(int scheme, int unit_draw, const double *rates, const int32_t *active, int count, double draw,
                int64_t *selected, double *bound) {
    /* Lifting.reset / insert (lifting.py:38-80): the negated negative derivatives and their table indices,
     * the random position from the positive derivatives up to and including the active unit */
    double *negative = (double *)malloc(sizeof(double) * (size_t)(count > 0 ? count : 1));
    int *where = (int *)malloc(sizeof(int) * (size_t)(count > 0 ? count : 1));
    int negatives = 0, active_recorded = 0, status = JFO_OK;
    double random_position = 0.0, uniform_bound = NAN;
    *selected = -1;
    for (int i = 0; i < count && status == JFO_OK; ++i) {
        if (rates[i] > 0.0) {
            if (active[i]) {
                if (active_recorded) {
                    status = JFO_ASSERT;  /* one active unit per table (lifting.py:33-34) */
                    break;
                }
                active_recorded = 1;
                uniform_bound = rates[i];
                random_position += unit_draw ? py_uniform(0.0, rates[i], draw) : draw;
            } else if (!active_recorded) {
                random_position += rates[i];
            }
        } else {
            if (active[i]) {
                status = JFO_ASSERT;  /* lifting.py:76 */
                break;
            }
            negative[negatives] = -rates[i];
            where[negatives] = i;
            ++negatives;
        }
    }
    if (status == JFO_OK && !active_recorded) status = JFO_LIFTING;  /* lifting.py:107-108 */
    if (status != JFO_OK) {
        *bound = NAN;
    } else {
        double total = jfo_py_sum(negative, negatives);
        double position = random_position;
        if (scheme == 1) {
            position = total - random_position;  /* outside_first_lifting.py:49 */
        } else if (scheme == 2) {
            uniform_bound = total;               /* ratio_lifting.py:50 */
            position = unit_draw ? py_uniform(0.0, total, draw) : draw;
        }
        *bound = uniform_bound;
        if (negatives == 0) {
            status = JFO_INDEX;                  /* identifiers[-1] of an empty list */
        } else {
            double summed = 0.0;
            *selected = where[negatives - 1];
            for (int k = 0; k < negatives; ++k) {
                summed += negative[k];
                if (position <= summed) {
                    *selected = where[k];
                    break;
                }
            }
        }
    }
    free(negative);
    free(where);
    return status;
}

void jfo_cell_bounds(double system_length, int m, double *cell_min, double *cell_max) {
    double side = system_length / m;
    for (int i = 0; i < m; ++i) {
        double lower = i * side;
        double upper = (i + 1) * side;
        if (lower > 0.0) {
            while ((long long)(lower / side) == i) lower = next_down(lower);
            while ((long long)(lower / side) < i) lower = next_up(lower);
        }
        while ((long long)(upper / side) == i) upper = next_up(upper);
        while ((long long)(upper / side) > i) upper = next_down(upper);
        cell_min[i] = lower;
        cell_max[i] = upper;
    }
}

/* ======================================================================================
 * Walker's alias table (event_handler/walker.py:53-130)
 * ==================================================================================== */
typedef struct {
    int item;
    double rate;
} WItem;

typedef struct {
    int size;
    double total_rate, mean_rate;
    int *first_item, *second_item; /* second_item = -1 for single-element entries */
    double *first_rate;
} Walker;

static int walker_build(Walker *w, const int *items, const double *rates, int n) {
    w->size = 0;
    w->total_rate = jfo_py_sum(rates, n);
    w->mean_rate = w->total_rate / n;
    w->first_item = (int *)malloc(sizeof(int) * (n + 1));
    w->second_item = (int *)malloc(sizeof(int) * (n + 1));
    w->first_rate = (double *)malloc(sizeof(double) * (n + 1));
    WItem *small = (WItem *)malloc(sizeof(WItem) * (n + 1));
    WItem *large = (WItem *)malloc(sizeof(WItem) * (n + 1));
    if (!w->first_item || !w->second_item || !w->first_rate || !small || !large) return JFO_ALLOC;
    int ns = 0, nl = 0;
    for (int i = 0; i < n; ++i) {
        if (!(rates[i] >= 0.0)) return JFO_ASSERT;
        WItem it = {items[i], rates[i]};
        if (rates[i] > w->mean_rate)
            large[nl++] = it;
        else
            small[ns++] = it;
    }
    while (ns && nl) {
        WItem s = small[--ns];
        WItem l = large[--nl];
        w->first_item[w->size] = s.item;
        w->first_rate[w->size] = s.rate;
        w->second_item[w->size] = l.item;
        w->size++;
        l.rate -= w->mean_rate - s.rate;
        if (l.rate < w->mean_rate)
            small[ns++] = l;
        else
            large[nl++] = l;
    }
    while (ns) {
        WItem s = small[--ns];
        double ratio = s.rate / w->mean_rate;
        if (!(1 - 1e-6 < ratio && ratio < 1 + 1e-6)) return JFO_ASSERT;
        w->first_item[w->size] = s.item;
        w->first_rate[w->size] = w->mean_rate;
        w->second_item[w->size] = -1;
        w->size++;
    }
    while (nl) {
        WItem l = large[--nl];
        double ratio = l.rate / w->mean_rate;
        if (!(1 - 1e-6 < ratio && ratio < 1 + 1e-6)) return JFO_ASSERT;
        w->first_item[w->size] = l.item;
        w->first_rate[w->size] = w->mean_rate;
        w->second_item[w->size] = -1;
        w->size++;
    }
    free(small);
    free(large);
    return JFO_OK;
}

static void walker_free(Walker *w) {
    free(w->first_item);
    free(w->second_item);
    free(w->first_rate);
}

/* Walker's alias table (walker.py:53-103) over n items, exported: first_item / first_rate / second_item [n]
 * (second_item -1 for an entry of one item), the total and the mean rate. */
int jfo_walker_table(const int *items, const double *rates, int n, int *first_item, double *first_rate,
                     int *second_item, double *total_rate, double *mean_rate) {
    if (n < 1) return JFO_BAD_CONFIG;
    Walker w;
    int st = walker_build(&w, items, rates, n);
    if (st == JFO_OK) {
        for (int k = 0; k < w.size; ++k) {
            first_item[k] = w.first_item[k];
            first_rate[k] = w.first_rate[k];
            second_item[k] = w.second_item[k];
        }
        *total_rate = w.total_rate;
        *mean_rate = w.mean_rate;
    }
    walker_free(&w);
    return st;
}

/* Walker.sample_cell (walker.py:105-122) with the table index random.choice returned and the value of
 * random.uniform(0.0, mean rate): the entry's first item when the value does not exceed its first rate. */
int jfo_walker_pick(const int *first_item, const double *first_rate, const int *second_item, int size, int choice,
                    double uniform) {
    if (choice < 0 || choice >= size) return -1;
    return uniform <= first_rate[choice] ? first_item[choice] : second_item[choice];
}

/* Walker.sample_cell: random.choice(table), then uniform(0, mean) <= first rate */
static int walker_sample(const Walker *w, uint64_t choice_bits, uint64_t uniform_bits) {
    int k = (int)jfo_randbelow(choice_bits, (uint32_t)w->size);
    double u = w->mean_rate * jfo_uniform(uniform_bits);
    if (u <= w->first_rate[k]) return w->first_item[k];
    return w->second_item[k];
}

/* ======================================================================================
 * Chain engine
 * ==================================================================================== */
struct JfoChain {
    JfoSystem sys;
    double *pos;     /* [n][3] */
    double *charge;  /* [n] */
    double side, half;
    int m, ncells;
    double *cmin, *cmax; /* per-axis exact cell bounds */
    int *rel;            /* [m][m]: relative_cell index along an axis, rel[c*m + r] */
    int *tra;            /* [m][m]: translate index along an axis, tra[c*m + r] */
    unsigned char *near_axis; /* [m]: axis offset residue is within the neighbour layers */
    /* occupancy (single_active_cell_occupancy.py) */
    int *occ;        /* [ncells][cap] */
    int *occ_count;  /* [ncells] */
    int cap;
    int *sur;        /* [ncells][n] surplus lists */
    int *sur_count;  /* [ncells] */
    int occ_active;  /* _active_unit_identifier (-1 = None) */
    int occ_cell;    /* _active_cell */
    /* lifting state */
    int active, direction;
    double ts_q, ts_r;
    double eoc_q, eoc_r;
    int eoc_new_active;
    int64_t event;
    /* excess displacement of the liftings (pressure estimator of the harness, not part of the reference) */
    double lift_sum;
    int64_t liftings;
    /* potentials */
    MH lj;
    MIC mic;
    int have_mic;
    /* far field tables */
    double *bound_upper;  /* [ncells][3] */
    double *bound_lower;  /* [ncells][3] (negated lower bound for the cell veto) */
    Walker walker[2][3];  /* [upper/lower][direction] */
    int have_walker;
    int64_t bound_warnings;
};

static int cell_of(const JfoChain *c, const double *p, int *cell) {
    long long ix = (long long)(p[0] / c->side), iy = (long long)(p[1] / c->side), iz = (long long)(p[2] / c->side);
    long long idx = ix + (long long)c->m * iy + (long long)c->m * c->m * iz;
    if (idx < 0 || idx >= c->ncells) return JFO_CELL_RANGE;
    *cell = (int)idx;
    return JFO_OK;
}

static void cell_axes(const JfoChain *c, int cell, int *a) {
    a[0] = cell % c->m;
    a[1] = (cell / c->m) % c->m;
    a[2] = cell / (c->m * c->m);
}

/* nearby_cells(cell) membership (cuboid_periodic_cells.py:74-100) */
static int is_nearby(const JfoChain *c, int cell, int reference) {
    int a[3], b[3];
    cell_axes(c, cell, a);
    cell_axes(c, reference, b);
    for (int d = 0; d < 3; ++d) {
        int diff = ((a[d] - b[d]) % c->m + c->m) % c->m;
        if (!c->near_axis[diff]) return 0;
    }
    return 1;
}

static int relative_cell(const JfoChain *c, int cell, int reference) {
    int a[3], b[3];
    cell_axes(c, cell, a);
    cell_axes(c, reference, b);
    return c->rel[a[0] * c->m + b[0]] + c->m * c->rel[a[1] * c->m + b[1]] +
           c->m * c->m * c->rel[a[2] * c->m + b[2]];
}

static int translate_cell(const JfoChain *c, int cell, int relative) {
    int a[3], b[3];
    cell_axes(c, cell, a);
    cell_axes(c, relative, b);
    return c->tra[a[0] * c->m + b[0]] + c->m * c->tra[a[1] * c->m + b[1]] +
           c->m * c->m * c->tra[a[2] * c->m + b[2]];
}

/* separation_vector (hypercubic_setting.py:120-172) */
static void separation(const JfoChain *c, const double *from, const double *to, double *s) {
    for (int d = 0; d < 3; ++d)
        s[d] = jfo_py_mod((to[d] - from[d]) + c->half, c->sys.system_length) - c->half;
}

/* InnerPointEstimator.derivative_bound (inner_point_estimator.py:108-163) */
static int estimator_bound(const JfoChain *c, const double *lower, const double *upper, int direction,
                           double *upper_out, double *lower_out) {
    int pps = c->sys.estimator_points;
    double ub = -INFINITY, lb = INFINITY;
    double velocity[3] = {0.0, 0.0, 0.0};
    velocity[direction] = 1.0;
    for (int ix = 0; ix < pps + 1; ++ix) {
        double px = lower[0] + ((upper[0] - lower[0]) * ix) / pps;
        for (int iy = 0; iy < pps + 1; ++iy) {
            double py = lower[1] + ((upper[1] - lower[1]) * iy) / pps;
            for (int iz = 0; iz < pps + 1; ++iz) {
                double pz = lower[2] + ((upper[2] - lower[2]) * iz) / pps;
                double s[3] = {px, py, pz};
                for (int d = 0; d < 3; ++d) s[d] = jfo_py_mod(s[d] + c->half, c->sys.system_length) - c->half;
                double derivative;
                if (c->sys.potential == JFO_POT_LENNARD_JONES) {
                    int st = mh_derivative(&c->lj, velocity, s, &derivative);
                    if (st) return st;
                } else {
                    derivative = mic_std_derivative(&c->mic, c->sys.coulomb_prefactor, direction, s, 1.0, 1.0) * 1.0;
                }
                /* max()/min() keep the first argument on ties and NaN comparisons */
                if (derivative > ub) ub = derivative;
                if (derivative < lb) lb = derivative;
            }
        }
    }
    double pref = c->sys.estimator_prefactor;
    if (ub > 0.0)
        ub *= pref;
    else
        ub /= pref;
    if (lb > 0.0)
        lb /= pref;
    else
        lb *= pref;
    *upper_out = ub; /* empirical bound is infinite */
    *lower_out = lb;
    return JFO_OK;
}

static int build_far_tables(JfoChain *c) {
    int ncells = c->ncells;
    c->bound_upper = (double *)calloc((size_t)ncells * 3, sizeof(double));
    c->bound_lower = (double *)calloc((size_t)ncells * 3, sizeof(double));
    if (!c->bound_upper || !c->bound_lower) return JFO_ALLOC;
    /* cell_bounding_potential.py:104-118 and cell_veto_event_handler.py:134-159: loop over the
     * cells that are not nearby the zero cell; the relative cell of such a cell to the zero cell
     * is the cell itself. */
    for (int cell = 0; cell < ncells; ++cell) {
        if (is_nearby(c, cell, 0)) continue;
        int a[3];
        cell_axes(c, cell, a);
        double lower[3], upper[3];
        for (int d = 0; d < 3; ++d) {
            lower[d] = c->cmin[a[d]] - c->cmax[0];
            upper[d] = c->cmax[a[d]] - c->cmin[0];
        }
        for (int d = 0; d < 3; ++d) {
            double ub, lb;
            int st = estimator_bound(c, lower, upper, d, &ub, &lb);
            if (st) return st;
            c->bound_upper[cell * 3 + d] = ub;
            c->bound_lower[cell * 3 + d] = -lb;
        }
    }
    if (c->sys.far == JFO_FAR_CELL_VETO) {
        int *items = (int *)malloc(sizeof(int) * ncells);
        double *rates = (double *)malloc(sizeof(double) * ncells);
        if (!items || !rates) return JFO_ALLOC;
        for (int which = 0; which < 2; ++which)
            for (int d = 0; d < 3; ++d) {
                int n = 0;
                for (int cell = 0; cell < ncells; ++cell) {
                    if (is_nearby(c, cell, 0)) continue;
                    double r = which == 0 ? c->bound_upper[cell * 3 + d] : c->bound_lower[cell * 3 + d];
                    items[n] = cell;
                    rates[n] = r > 0.0 ? r : 0.0; /* max(bound, 0.0) */
                    ++n;
                }
                int st = walker_build(&c->walker[which][d], items, rates, n);
                if (st) return st;
            }
        c->have_walker = 1;
        free(items);
        free(rates);
    }
    return JFO_OK;
}

static void occ_insert(JfoChain *c, int cell, int id) {
    if (c->occ_count[cell] < c->cap) {
        c->occ[cell * c->cap + c->occ_count[cell]++] = id;
    } else {
        c->sur[(size_t)cell * c->sys.n + c->sur_count[cell]++] = id;
    }
}

/* list.remove: first occurrence, order of the rest kept */
static int list_remove(int *list, int *count, int id) {
    for (int i = 0; i < *count; ++i)
        if (list[i] == id) {
            for (int k = i + 1; k < *count; ++k) list[k - 1] = list[k];
            --*count;
            return 1;
        }
    return 0;
}

/* SingleActiveCellOccupancy.update (single_active_cell_occupancy.py:149-203) */
static int occ_update(JfoChain *c) {
    int st;
    if (c->active != c->occ_active) {
        if (c->occ_active >= 0) occ_insert(c, c->occ_cell, c->occ_active);
        st = cell_of(c, &c->pos[3 * c->active], &c->occ_cell);
        if (st) return st;
        c->occ_active = c->active;
        if (!list_remove(&c->occ[c->occ_cell * c->cap], &c->occ_count[c->occ_cell], c->active)) {
            if (!list_remove(&c->sur[(size_t)c->occ_cell * c->sys.n], &c->sur_count[c->occ_cell], c->active))
                return JFO_ASSERT;
        }
    } else {
        st = cell_of(c, &c->pos[3 * c->active], &c->occ_cell);
        if (st) return st;
    }
    return JFO_OK;
}

JfoChain *jfo_chain_create(const JfoSystem *system, const double *positions, const double *charges, int *status) {
    *status = JFO_OK;
    JfoChain *c = (JfoChain *)calloc(1, sizeof(JfoChain));
    if (!c) {
        *status = JFO_ALLOC;
        return NULL;
    }
    c->sys = *system;
    int n = system->n, m = system->cells_per_side;
    if (n < 2 || m < 1 || system->max_occupants < 1 || !(system->system_length > 0.0) ||
        system->initial_active < 0 || system->initial_active >= n || system->initial_direction < 0 ||
        system->initial_direction > 2 || !(system->speed > 0.0)) {
        *status = JFO_BAD_CONFIG;
        free(c);
        return NULL;
    }
    c->m = m;
    c->ncells = m * m * m;
    c->side = system->system_length / m;
    c->half = system->system_length / 2.0;
    c->cap = system->max_occupants;
    c->pos = (double *)malloc(sizeof(double) * 3 * n);
    c->charge = (double *)malloc(sizeof(double) * n);
    c->cmin = (double *)malloc(sizeof(double) * m);
    c->cmax = (double *)malloc(sizeof(double) * m);
    c->rel = (int *)malloc(sizeof(int) * m * m);
    c->tra = (int *)malloc(sizeof(int) * m * m);
    c->near_axis = (unsigned char *)calloc(m, 1);
    c->occ = (int *)malloc(sizeof(int) * c->ncells * c->cap);
    c->occ_count = (int *)calloc(c->ncells, sizeof(int));
    c->sur = (int *)malloc(sizeof(int) * (size_t)c->ncells * n);
    c->sur_count = (int *)calloc(c->ncells, sizeof(int));
    if (!c->pos || !c->charge || !c->cmin || !c->cmax || !c->rel || !c->tra || !c->near_axis || !c->occ ||
        !c->occ_count || !c->sur || !c->sur_count) {
        *status = JFO_ALLOC;
        jfo_chain_destroy(c);
        return NULL;
    }
    memcpy(c->pos, positions, sizeof(double) * 3 * n);
    for (int i = 0; i < n; ++i) c->charge[i] = charges ? charges[i] : 1.0;
    jfo_cell_bounds(system->system_length, m, c->cmin, c->cmax);
    for (int o = -system->neighbor_layers; o <= system->neighbor_layers; ++o) c->near_axis[((o % m) + m) % m] = 1;
    /* relative_cell / translate along one axis (cuboid_periodic_cells.py:156-207) */
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < m; ++b) {
            double center = (c->cmax[a] + c->cmin[a]) / 2.0;
            double r = jfo_py_mod(center - c->cmin[b], system->system_length);
            double t = jfo_py_mod(center + c->cmin[b], system->system_length);
            c->rel[a * m + b] = (int)(long long)(r / c->side);
            c->tra[a * m + b] = (int)(long long)(t / c->side);
        }
    if (system->potential == JFO_POT_LENNARD_JONES) c->lj = mh_lj(system->lj_prefactor, system->lj_sigma);
    if (system->potential == JFO_POT_COULOMB) {
        if (mic_init(&c->mic, system->fourier_cutoff, system->position_cutoff, system->ewald_alpha,
                     system->system_length)) {
            *status = JFO_ALLOC;
            jfo_chain_destroy(c);
            return NULL;
        }
        c->have_mic = 1;
    }
    /* SingleActiveCellOccupancy.initialize (single_active_cell_occupancy.py:95-121) */
    for (int i = 0; i < n; ++i) {
        int cell;
        int st = cell_of(c, &c->pos[3 * i], &cell);
        if (st) {
            *status = st;
            jfo_chain_destroy(c);
            return NULL;
        }
        occ_insert(c, cell, i);
    }
    c->occ_active = -1;
    c->occ_cell = -1;
    if (system->far != JFO_FAR_NONE) {
        if ((system->far == JFO_FAR_CELL_VETO || system->far == JFO_FAR_CELL_BOUNDING) && c->cap != 1) {
            *status = JFO_BAD_CONFIG;
            jfo_chain_destroy(c);
            return NULL;
        }
        int st = build_far_tables(c);
        if (st) {
            *status = st;
            jfo_chain_destroy(c);
            return NULL;
        }
    }
    /* InitialChainStartOfRunEventHandler (initial_chain_start_of_run_event_handler.py): time stamp 0 */
    c->active = system->initial_active;
    c->direction = system->initial_direction;
    c->ts_q = 0.0;
    c->ts_r = 0.0;
    c->event = 0;
    /* first end-of-chain candidate: Time(0, 0) + ((Time(0, 0) - Time(0, 0)) + chain_time) */
    jfo_time_add(0.0, 0.0, jfo_time_sub(0.0, 0.0, 0.0, 0.0) + system->chain_time, &c->eoc_q, &c->eoc_r);
    c->eoc_new_active = (int)jfo_randbelow(jfo_draw(system->rng_key, 0, JFO_RNG_NEW_ACTIVE, 0), (uint32_t)n);
    return c;
}

void jfo_chain_destroy(JfoChain *c) {
    if (!c) return;
    free(c->pos);
    free(c->charge);
    free(c->cmin);
    free(c->cmax);
    free(c->rel);
    free(c->tra);
    free(c->near_axis);
    free(c->occ);
    free(c->occ_count);
    free(c->sur);
    free(c->sur_count);
    free(c->bound_upper);
    free(c->bound_lower);
    if (c->have_mic) free(c->mic.fourier);
    if (c->have_walker)
        for (int w = 0; w < 2; ++w)
            for (int d = 0; d < 3; ++d) walker_free(&c->walker[w][d]);
    free(c);
}

typedef struct {
    double q, r;
    int kind, target;
    int aux; /* cell-veto target cell / cell-bounding relative cell */
    double rate;
} Cand;

/* Candidate order: the earliest time first; on equal times the lower kind, then the lower target.
 * (The reference heap breaks exact ties by insertion order; continuous random potential changes
 * make exact ties of distinct candidates an event of probability zero.) */
static int cand_better(const Cand *a, const Cand *b) {
    if (jfo_time_lt(a->q, a->r, b->q, b->r)) return 1;
    if (jfo_time_lt(b->q, b->r, a->q, a->r)) return 0;
    if (a->kind != b->kind) return a->kind < b->kind;
    return a->target < b->target;
}

static void offer(Cand *best, double ts_q, double ts_r, double dt, int kind, int target, int aux, double rate) {
    if (isinf(dt) && dt > 0) return; /* HeapScheduler.push_event ignores infinite times */
    Cand c;
    jfo_time_add(ts_q, ts_r, dt, &c.q, &c.r);
    c.kind = kind;
    c.target = target;
    c.aux = aux;
    c.rate = rate;
    if (cand_better(&c, best)) *best = c;
}

/* candidates of one pair (active, target) from the nearby/surplus taggers */
static int pair_candidates(JfoChain *c, int target, Cand *best) {
    const JfoSystem *s = &c->sys;
    double sep[3], velocity[3] = {0.0, 0.0, 0.0}, dt;
    velocity[c->direction] = s->speed;
    separation(c, &c->pos[3 * c->active], &c->pos[3 * target], sep);
    int st;
    if (s->potential == JFO_POT_HARD_SPHERE) {
        /* TwoLeafUnitEventHandler with HardSpherePotential (no potential change) */
        st = jfo_hs_displacement(s->hs_radius, velocity, sep, &dt);
        if (st) return st;
        offer(best, c->ts_q, c->ts_r, dt, JFO_EV_PAIR, target, -1, 0.0);
    } else if (s->potential == JFO_POT_LENNARD_JONES) {
        /* two_leaf_unit_event_handler.py:98-138 */
        double du = jfo_expovariate(jfo_draw(s->rng_key, c->event, JFO_RNG_PAIR, target), s->beta);
        st = mh_displacement(&c->lj, velocity, sep, du, &dt);
        if (st) return st;
        offer(best, c->ts_q, c->ts_r, dt, JFO_EV_PAIR, target, -1, 0.0);
    } else {
        if (s->hs_radius > 0.0) {
            st = jfo_hs_displacement(s->hs_radius, velocity, sep, &dt);
            if (st) return st;
            offer(best, c->ts_q, c->ts_r, dt, JFO_EV_HARDCORE, target, -1, 0.0);
        }
        /* two_leaf_unit_bounding_potential_event_handler.py:112-143 */
        double du = jfo_expovariate(jfo_draw(s->rng_key, c->event, JFO_RNG_PAIR, target), s->beta);
        st = jfo_ipcb_displacement(s->bound_prefactor, s->system_length, velocity, sep, c->charge[c->active],
                                   c->charge[target], du, &dt);
        if (st) return st;
        offer(best, c->ts_q, c->ts_r, dt, JFO_EV_BOUNDED, target, -1, 0.0);
    }
    return JFO_OK;
}

static void time_slice_active(JfoChain *c, double q, double r) {
    double dt = jfo_time_sub(q, r, c->ts_q, c->ts_r);
    double *p = &c->pos[3 * c->active];
    for (int d = 0; d < 3; ++d) {
        double v = d == c->direction ? c->sys.speed : 0.0;
        p[d] = jfo_py_mod(p[d] + v * dt, c->sys.system_length);
    }
    c->ts_q = q;
    c->ts_r = r;
}

/* real derivative of the thinning decision (event_handler_with_bounding_potential.py:75-101) */
static int real_derivative(JfoChain *c, int target, double *out) {
    double sep[3], velocity[3] = {0.0, 0.0, 0.0};
    velocity[c->direction] = c->sys.speed;
    separation(c, &c->pos[3 * c->active], &c->pos[3 * target], sep);
    if (c->sys.potential == JFO_POT_LENNARD_JONES) return mh_derivative(&c->lj, velocity, sep, out);
    *out = mic_std_derivative(&c->mic, c->sys.coulomb_prefactor, c->direction, sep, c->charge[c->active],
                              c->charge[target]) *
           c->sys.speed;
    return JFO_OK;
}

static int thinning(JfoChain *c, int target, double bounding_rate, int *accepted) {
    double real;
    int st = real_derivative(c, target, &real);
    if (st) return st;
    *accepted = 0;
    if (real > 0) {
        if (bounding_rate < real) c->bound_warnings++;
        double u = bounding_rate * jfo_uniform(jfo_draw(c->sys.rng_key, c->event, JFO_RNG_THIN, 0));
        if (u < real) *accepted = 1;
    }
    return JFO_OK;
}

int64_t jfo_chain_run(JfoChain *c, int64_t max_events, double stop_q, double stop_r, JfoEvent *log,
                      int *status) {
    const JfoSystem *s = &c->sys;
    int64_t done = 0;
    *status = JFO_OK;
    int st;
    while (done < max_events) {
        st = occ_update(c);
        if (st) {
            *status = st;
            return done;
        }
        Cand best;
        best.q = INFINITY;
        best.r = INFINITY;
        best.kind = 1 << 30;
        best.target = 1 << 30;
        best.aux = -1;
        best.rate = 0.0;
        /* ExcludedCellsTagger: occupants of the nearby cells of the active cell */
        int a[3];
        cell_axes(c, c->occ_cell, a);
        int n_off = 0, offsets[64];
        for (int o = 0; o < c->m; ++o)
            if (c->near_axis[o]) offsets[n_off++] = o;
        for (int oz = 0; oz < n_off; ++oz)
            for (int oy = 0; oy < n_off; ++oy)
                for (int ox = 0; ox < n_off; ++ox) {
                    int cell = (a[0] + offsets[ox]) % c->m + c->m * ((a[1] + offsets[oy]) % c->m) +
                               c->m * c->m * ((a[2] + offsets[oz]) % c->m);
                    for (int k = 0; k < c->occ_count[cell]; ++k) {
                        st = pair_candidates(c, c->occ[cell * c->cap + k], &best);
                        if (st) {
                            *status = st;
                            return done;
                        }
                    }
                }
        /* SurplusCellsTagger */
        for (int cell = 0; cell < c->ncells; ++cell)
            for (int k = 0; k < c->sur_count[cell]; ++k) {
                st = pair_candidates(c, c->sur[(size_t)cell * s->n + k], &best);
                if (st) {
                    *status = st;
                    return done;
                }
            }
        int active_cell;
        st = cell_of(c, &c->pos[3 * c->active], &active_cell);
        if (st) {
            *status = st;
            return done;
        }
        double velocity_speed = s->speed;
        if (s->far == JFO_FAR_CELL_BOUNDING) {
            /* CellBoundingPotentialTagger + TwoLeafUnitCellBoundingPotentialEventHandler */
            for (int cell = 0; cell < c->ncells; ++cell) {
                if (c->occ_count[cell] == 0 || is_nearby(c, cell, c->occ_cell)) continue;
                int target = c->occ[cell * c->cap];
                int target_cell;
                st = cell_of(c, &c->pos[3 * target], &target_cell);
                if (st) {
                    *status = st;
                    return done;
                }
                int rc = relative_cell(c, target_cell, active_cell);
                double du = jfo_expovariate(jfo_draw(s->rng_key, c->event, JFO_RNG_PAIR, target), s->beta);
                double rate = c->bound_upper[rc * 3 + c->direction];
                double disp = rate > 0 ? du / rate : INFINITY;
                offer(&best, c->ts_q, c->ts_r, disp / velocity_speed, JFO_EV_CELL_BOUNDING, target, rc, rate);
            }
        } else if (s->far == JFO_FAR_CELL_VETO) {
            /* CellVetoEventHandler.send_event_time (cell_veto_event_handler.py:162-238) */
            double charge_factor = c->charge[c->active] * 1.0 / 1.0;
            int which = 0;
            if (s->potential == JFO_POT_LENNARD_JONES) charge_factor = 1.0;
            if (!(charge_factor > 0.0)) {
                charge_factor *= -1.0;
                which = 1;
            }
            const Walker *w = &c->walker[which][c->direction];
            double total_rate = w->total_rate * charge_factor;
            int rc = walker_sample(w, jfo_draw(s->rng_key, c->event, JFO_RNG_VETO_CHOICE, 0),
                                   jfo_draw(s->rng_key, c->event, JFO_RNG_VETO_UNIFORM, 0));
            double rate = (which == 0 ? c->bound_upper[rc * 3 + c->direction] : c->bound_lower[rc * 3 + c->direction]) *
                          charge_factor;
            if (!(rate > 0.0)) {
                *status = JFO_ASSERT;
                return done;
            }
            int target_cell = translate_cell(c, active_cell, rc);
            double dt = jfo_expovariate(jfo_draw(s->rng_key, c->event, JFO_RNG_VETO_TIME, 0), s->beta) /
                        (total_rate * velocity_speed);
            offer(&best, c->ts_q, c->ts_r, dt, JFO_EV_CELL_VETO, -1, target_cell, rate);
        }
        /* CellBoundaryEventHandler.send_event_time (cell_boundary_event_handler.py:98-156) */
        {
            int ax[3];
            cell_axes(c, active_cell, ax);
            int d = c->direction;
            double boundary = c->cmin[(ax[d] + 1) % c->m];
            double sep = boundary - c->pos[3 * c->active + d];
            if (sep < 0.0) sep = sep + s->system_length;
            offer(&best, c->ts_q, c->ts_r, sep / s->speed, JFO_EV_BOUNDARY, -1, -1, boundary);
        }
        /* end of chain (persistent candidate) */
        {
            Cand e;
            e.q = c->eoc_q;
            e.r = c->eoc_r;
            e.kind = JFO_EV_END_OF_CHAIN;
            e.target = c->eoc_new_active;
            e.aux = -1;
            e.rate = 0.0;
            if (cand_better(&e, &best)) best = e;
        }
        /* stop time: wins ties */
        if (!isinf(stop_q) && !jfo_time_lt(best.q, best.r, stop_q, stop_r)) {
            time_slice_active(c, stop_q, stop_r);
            return done;
        }
        /* commit */
        JfoEvent ev;
        ev.kind = best.kind;
        ev.moved = c->active;
        ev.target = -1;
        ev.accepted = 0;
        ev.time_q = best.q;
        ev.time_r = best.r;
        time_slice_active(c, best.q, best.r);
        int moved = c->active;
        switch (best.kind) {
        case JFO_EV_PAIR:
        case JFO_EV_HARDCORE:
            ev.target = best.target;
            ev.accepted = 1;
            c->active = best.target;
            break;
        case JFO_EV_BOUNDED: {
            /* out-state: IPCB derivative at the event time, then thinning with the merged image */
            double sep[3], velocity[3] = {0.0, 0.0, 0.0}, bound;
            velocity[c->direction] = s->speed;
            separation(c, &c->pos[3 * c->active], &c->pos[3 * best.target], sep);
            st = jfo_ipcb_derivative(s->bound_prefactor, velocity, sep, c->charge[c->active],
                                     c->charge[best.target], &bound);
            if (st) {
                *status = st;
                return done;
            }
            int accepted;
            st = thinning(c, best.target, bound, &accepted);
            if (st) {
                *status = st;
                return done;
            }
            ev.target = best.target;
            ev.accepted = accepted;
            if (accepted) c->active = best.target;
            break;
        }
        case JFO_EV_CELL_BOUNDING: {
            int now_cell;
            st = cell_of(c, &c->pos[3 * c->active], &now_cell);
            if (st || now_cell != active_cell) {
                *status = st ? st : JFO_ASSERT;
                return done;
            }
            int accepted;
            st = thinning(c, best.target, best.rate * s->speed, &accepted);
            if (st) {
                *status = st;
                return done;
            }
            ev.target = best.target;
            ev.accepted = accepted;
            if (accepted) c->active = best.target;
            break;
        }
        case JFO_EV_CELL_VETO: {
            int cell = best.aux;
            if (c->occ_count[cell] > 0) {
                int target = c->occ[cell * c->cap];
                int accepted;
                st = thinning(c, target, best.rate, &accepted);
                if (st) {
                    *status = st;
                    return done;
                }
                ev.target = target;
                ev.accepted = accepted;
                if (accepted) c->active = target;
            }
            break;
        }
        case JFO_EV_BOUNDARY:
            c->pos[3 * c->active + c->direction] = best.rate;
            break;
        case JFO_EV_END_OF_CHAIN: {
            c->direction = (c->direction + 1) % 3;
            c->active = best.target;
            ev.target = best.target;
            ev.accepted = 1;
            /* next end-of-chain candidate, created in the next loop iteration */
            jfo_time_add(c->ts_q, c->ts_r, jfo_time_sub(c->ts_q, c->ts_r, c->ts_q, c->ts_r) + s->chain_time,
                         &c->eoc_q, &c->eoc_r);
            c->eoc_new_active =
                (int)jfo_randbelow(jfo_draw(s->rng_key, (uint64_t)(c->event + 1), JFO_RNG_NEW_ACTIVE, 0),
                                   (uint32_t)s->n);
            break;
        }
        default:
            *status = JFO_ASSERT;
            return done;
        }
        if (c->active != moved && best.kind != JFO_EV_END_OF_CHAIN) {
            /* separation target - active along the direction of motion, as separation_vector computes it */
            int d = c->direction;
            c->lift_sum += jfo_py_mod((c->pos[3 * c->active + d] - c->pos[3 * moved + d]) + c->half,
                                      s->system_length) - c->half;
            c->liftings++;
        }
        ev.new_active = c->active;
        ev.new_direction = c->direction;
        ev.x = c->pos[3 * moved];
        ev.y = c->pos[3 * moved + 1];
        ev.z = c->pos[3 * moved + 2];
        if (log) log[done] = ev;
        c->event++;
        done++;
    }
    return done;
}

void jfo_chain_positions(const JfoChain *c, double *positions) {
    memcpy(positions, c->pos, sizeof(double) * 3 * c->sys.n);
}

void jfo_chain_state(const JfoChain *c, int64_t *event_count, int *active, int *direction, double *time_q,
                     double *time_r) {
    *event_count = c->event;
    *active = c->active;
    *direction = c->direction;
    *time_q = c->ts_q;
    *time_r = c->ts_r;
}

void jfo_chain_liftings(const JfoChain *c, double *lift_sum, int64_t *liftings) {
    *lift_sum = c->lift_sum;
    *liftings = c->liftings;
}

/* far-field bound table: [ncells][3] upper bounds followed by [ncells][3] negated lower bounds */
int jfo_chain_bounds(const JfoChain *c, double *bounds, int capacity) {
    int need = c->ncells * 6;
    if (!c->bound_upper || capacity < need) return -need;
    memcpy(bounds, c->bound_upper, sizeof(double) * c->ncells * 3);
    memcpy(bounds + c->ncells * 3, c->bound_lower, sizeof(double) * c->ncells * 3);
    return need;
}

/* Walker table of the cell veto: entries (first cell, first rate, second cell) */
int jfo_chain_walker(const JfoChain *c, int direction, int which, int32_t *cells, double *rates, int capacity,
                     double *total_rate) {
    if (!c->have_walker) return -1;
    const Walker *w = &c->walker[which][direction];
    if (capacity < w->size) return -w->size;
    for (int i = 0; i < w->size; ++i) {
        cells[2 * i] = w->first_item[i];
        cells[2 * i + 1] = w->second_item[i];
        rates[i] = w->first_rate[i];
    }
    *total_rate = w->total_rate;
    return w->size;
}

/* occupancy snapshot for checks: owner[i] = cell of particle i in the occupants (>= 0), -2 - cell when it is a
 * surplus unit, -1 when it is the occupancy's active unit; returns the occupancy's active cell */
int jfo_chain_occupancy(const JfoChain *c, int32_t *owner) {
    for (int i = 0; i < c->sys.n; ++i) owner[i] = -100;
    for (int cell = 0; cell < c->ncells; ++cell) {
        for (int k = 0; k < c->occ_count[cell]; ++k) owner[c->occ[cell * c->cap + k]] = cell;
        for (int k = 0; k < c->sur_count[cell]; ++k) owner[c->sur[(size_t)cell * c->sys.n + k]] = -2 - cell;
    }
    if (c->occ_active >= 0) owner[c->occ_active] = -1;
    return c->occ_cell;
}

/* ======================================================================================
 * Flexible water (composite objects): the reference's event loop over the factors of a factor-set file
 * (two_leaf_unit_event_handler.py:98-154 for the bonds and Lennard-Jones, the composite-object Coulomb factor of
 * two_composite_object_summed_bounding_potential_event_handler.py:119-202, the end of chain of
 * single_independent_active_periodic_direction_end_of_chain_event_handler.py:151-237)
 * ==================================================================================== */
struct JfoWater {
    JfoWaterSystem sys;
    int units;
    double *pos;
    double *charge;
    MH oh, hh, lj;
    int active, direction;
    double ts_q, ts_r;      /* time stamp of the active unit */
    double eoc_q, eoc_r;    /* end-of-chain candidate */
    int eoc_new_active;
    int64_t event;
    /* molecular cells (NULL: a Coulomb factor with every other molecule): the cell system, occupancy and cell-veto
     * tables of the root units, whose positions the chain holds (cells->pos, [M][3]); cells->active is the active
     * molecule */
    JfoChain *cells;
    double root_speed;      /* the active root unit's velocity component: the leaf's times its weight 1/3 */
    /* the bond and Lennard-Jones candidates persist across molecular cell-boundary events: their earliest, and the
     * active leaf and root unit as their in-state holds them (time stamp snap_q, snap_r) */
    int keep_pairs;         /* the cell boundary trashes only the cell-based factors */
    int far;                /* JFO_FAR_CELL_VETO or JFO_FAR_CELL_BOUNDING (one candidate per occupied far cell) */
    double dipole_charge;   /* the dipole estimator's charge (the cell-bounding charge factor) */
    int pairs_valid;
    Cand pair;
    double snap_leaf[3], snap_root[3], snap_q, snap_r;
};

static int water_new_active(const JfoWater *w, uint64_t event) {
    int molecule = (int)jfo_randbelow(jfo_draw(w->sys.rng_key, event, JFO_RNG_NEW_ACTIVE, 0),
                                      (uint32_t)w->sys.molecules);
    int unit = (int)jfo_randbelow(jfo_draw(w->sys.rng_key, event, JFO_RNG_NEW_ACTIVE, 1), 3u);
    return 3 * molecule + unit;
}

JfoWater *jfo_water_create(const JfoWaterSystem *system, const double *positions, const double *charges,
                           int *status) {
    *status = JFO_BAD_CONFIG;
    if (system->molecules < 2 || !(system->system_length > 0.0) || system->initial_active < 0 ||
        system->initial_active >= 3 * system->molecules || system->lifting < 0 || system->lifting > 2)
        return NULL;
    JfoWater *w = (JfoWater *)calloc(1, sizeof(JfoWater));
    if (!w) {
        *status = JFO_ALLOC;
        return NULL;
    }
    w->sys = *system;
    w->units = 3 * system->molecules;
    w->pos = (double *)malloc(sizeof(double) * 3 * (size_t)w->units);
    w->charge = (double *)malloc(sizeof(double) * (size_t)w->units);
    if (!w->pos || !w->charge) {
        jfo_water_destroy(w);
        *status = JFO_ALLOC;
        return NULL;
    }
    memcpy(w->pos, positions, sizeof(double) * 3 * (size_t)w->units);
    memcpy(w->charge, charges, sizeof(double) * (size_t)w->units);
    w->oh = mh_dep(system->oh_r0, 2, system->oh_prefactor);
    w->hh = mh_dep(system->hh_r0, 2, system->hh_prefactor);
    w->lj = mh_lj(system->lj_prefactor, system->lj_sigma);
    w->active = system->initial_active;
    w->direction = system->initial_direction;
    w->ts_q = 0.0;
    w->ts_r = 0.0;
    jfo_time_add(0.0, 0.0, jfo_time_sub(0.0, 0.0, 0.0, 0.0) + system->chain_time, &w->eoc_q, &w->eoc_r);
    w->eoc_new_active = water_new_active(w, 0);
    *status = JFO_OK;
    return w;
}

void jfo_water_destroy(JfoWater *w) {
    if (!w) return;
    jfo_chain_destroy(w->cells);
    free(w->pos);
    free(w->charge);
    free(w);
}

static void water_separation(const JfoWater *w, int from, int to, double *s) {
    composite_separation(w->sys.system_length, &w->pos[3 * from], &w->pos[3 * to], s);
}

static int64_t water_cells_run(JfoWater *w, int64_t max_events, JfoEvent *log, double *root_log, int *status);

int64_t jfo_water_run(JfoWater *w, int64_t max_events, JfoEvent *log, int *status) {
    return jfo_water_run_roots(w, max_events, log, NULL, status);
}

int64_t jfo_water_run_roots(JfoWater *w, int64_t max_events, JfoEvent *log, double *root_log, int *status) {
    if (w->cells) return water_cells_run(w, max_events, log, root_log, status);
    const JfoWaterSystem *s = &w->sys;
    const int M = s->molecules;
    int64_t done = 0;
    *status = JFO_OK;
    while (done < max_events) {
        const int a = w->active, m = a / 3, t = a % 3;
        double velocity[3] = {0.0, 0.0, 0.0};
        velocity[w->direction] = s->speed;
        Cand best;
        best.q = INFINITY;
        best.r = INFINITY;
        best.kind = 1 << 30;
        best.target = 1 << 30;
        best.aux = -1;
        best.rate = 0.0;
        int st = JFO_OK;
        /* bonds of the active unit's molecule: O-H for pairs with the oxygen, H-H between the hydrogens */
        for (int u = 0; u < 3 && !st; ++u) {
            if (u == t) continue;
            const MH *bond = (t == 1 || u == 1) ? &w->oh : &w->hh;
            int b = 3 * m + u;
            double sep[3], dt;
            water_separation(w, a, b, sep);
            double du = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_PAIR, b), s->beta);
            st = mh_displacement(bond, velocity, sep, du, &dt);
            if (!st) offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_BOND, b, -1, 0.0);
        }
        /* Lennard-Jones between the active oxygen and every other oxygen */
        for (int other = 0; other < M && !st && t == 1; ++other) {
            if (other == m) continue;
            int b = 3 * other + 1;
            double sep[3], dt;
            water_separation(w, a, b, sep);
            double du = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_PAIR, b), s->beta);
            st = mh_displacement(&w->lj, velocity, sep, du, &dt);
            if (!st) offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_PAIR, b, -1, 0.0);
        }
        /* Coulomb factor of the active molecule with every other molecule */
        for (int other = 0; other < M && !st; ++other) {
            if (other == m) continue;
            double du[3], dt;
            for (int j = 0; j < 3; ++j)
                du[j] = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_COMPOSITE, (uint32_t)(3 * other + j)),
                                        s->beta);
            st = jfo_composite_event_time(3, s->ewald_alpha, s->fourier_cutoff, s->position_cutoff,
                                          s->coulomb_prefactor, s->bound_prefactor, s->system_length, velocity,
                                          &w->pos[3 * a], w->charge[a], &w->pos[9 * other], &w->charge[3 * other], du,
                                          &dt);
            if (!st) offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_COMPOSITE, other, -1, 0.0);
        }
        if (st) {
            *status = st;
            return done;
        }
        {
            Cand e;
            e.q = w->eoc_q;
            e.r = w->eoc_r;
            e.kind = JFO_EV_END_OF_CHAIN;
            e.target = w->eoc_new_active;
            e.aux = -1;
            e.rate = 0.0;
            if (cand_better(&e, &best)) best = e;
        }
        /* commit: time slice of the active unit, then the out-state */
        JfoEvent ev;
        ev.kind = best.kind;
        ev.moved = a;
        ev.target = best.target;
        ev.accepted = 1;
        ev.time_q = best.q;
        ev.time_r = best.r;
        {
            double dt = jfo_time_sub(best.q, best.r, w->ts_q, w->ts_r);
            double *p = &w->pos[3 * a];
            for (int d = 0; d < 3; ++d) {
                double v = d == w->direction ? s->speed : 0.0;
                p[d] = jfo_py_mod(p[d] + v * dt, s->system_length);
            }
            w->ts_q = best.q;
            w->ts_r = best.r;
        }
        switch (best.kind) {
        case JFO_EV_BOND:
        case JFO_EV_PAIR:
            w->active = best.target;
            break;
        case JFO_EV_COMPOSITE: {
            int other = best.target, new_active;
            double draws[3], bounding, rate;
            draws[0] = jfo_uniform(jfo_draw(s->rng_key, w->event, JFO_RNG_THIN, 0));
            draws[1] = jfo_uniform(jfo_draw(s->rng_key, w->event, JFO_RNG_LIFT, 0));
            draws[2] = draws[1];
            st = jfo_composite_out_state(3, s->lifting, 1, s->ewald_alpha, s->fourier_cutoff, s->position_cutoff,
                                         s->coulomb_prefactor, s->bound_prefactor, s->system_length, velocity,
                                         &w->pos[9 * m], &w->charge[3 * m], t, &w->pos[9 * other],
                                         &w->charge[3 * other], m < other, draws, &new_active, &bounding, &rate);
            if (st) {
                *status = st;
                return done;
            }
            ev.accepted = new_active >= 0;
            if (new_active >= 0) w->active = new_active < 3 ? 3 * m + new_active : 3 * other + (new_active - 3);
            break;
        }
        case JFO_EV_END_OF_CHAIN:
            w->direction = (w->direction + 1) % 3;
            w->active = best.target;
            jfo_time_add(w->ts_q, w->ts_r, jfo_time_sub(w->ts_q, w->ts_r, w->ts_q, w->ts_r) + s->chain_time,
                         &w->eoc_q, &w->eoc_r);
            w->eoc_new_active = water_new_active(w, (uint64_t)(w->event + 1));
            break;
        default:
            *status = JFO_ASSERT;
            return done;
        }
        ev.new_active = w->active;
        ev.new_direction = w->direction;
        ev.x = w->pos[3 * a];
        ev.y = w->pos[3 * a + 1];
        ev.z = w->pos[3 * a + 2];
        if (log) log[done] = ev;
        w->event++;
        done++;
    }
    return done;
}

/* ======================================================================================
 * Water with molecular cells: the Coulomb interaction of the active molecule by cells of root units
 * (SingleActiveCellOccupancy with cell_level 1, single_active_cell_occupancy.py:95-203): the summed-bounding factor
 * with the molecules of the nearby cells (ExcludedCellsTagger, excluded_cells_tagger.py:107-132) and with the
 * surplus molecules (SurplusCellsTagger, surplus_cells_tagger.py:107-131), the molecular cell veto
 * (CompositeObjectCellVetoEventHandler, composite_object_cell_veto_event_handler.py:110-162 with
 * abstracts/cell_veto_event_handler.py:162-238) and the cell-boundary event of the active root unit
 * (CellBoundaryEventHandler, cell_boundary_event_handler.py:98-173), whose tagger trashes and creates only the
 * cell-based factors: the bond and Lennard-Jones candidates persist across it.
 *
 * The root unit of the active molecule moves with the active leaf unit's velocity times the leaf's weight 1/3
 * (LeavesEventHandler._register_velocity_change_leaf_cnode / _commit_non_leaf_velocity_changes,
 * event_handler/abstracts/abstracts.py:165-234) and carries the leaf's time stamp; every committed out-state holds
 * it time-sliced to the event time (BasicEventHandler._time_slice_unit, abstracts.py:82-95).  A persistent bond or
 * Lennard-Jones candidate commits the copies its in-state took when it was created (tree_state_handler.py:104-145),
 * time-sliced from then to its event time, over the positions the cell-boundary events wrote meanwhile.
 * ==================================================================================== */

/* the bound tables of the molecular cell veto ([cells][3] upper, [cells][3] negated lower, as the estimator filled
 * CellVetoEventHandler._derivative_bounds; NaN for the nearby cells) and their Walker tables
 * (cell_veto_event_handler.py:134-160) */
static int chain_install_bounds(JfoChain *c, const double *upper, const double *lower) {
    int ncells = c->ncells;
    c->bound_upper = (double *)calloc((size_t)ncells * 3, sizeof(double));
    c->bound_lower = (double *)calloc((size_t)ncells * 3, sizeof(double));
    int *items = (int *)malloc(sizeof(int) * ncells);
    double *rates = (double *)malloc(sizeof(double) * ncells);
    if (!c->bound_upper || !c->bound_lower || !items || !rates) {
        free(items);
        free(rates);
        return JFO_ALLOC;
    }
    memcpy(c->bound_upper, upper, sizeof(double) * (size_t)ncells * 3);
    memcpy(c->bound_lower, lower, sizeof(double) * (size_t)ncells * 3);
    int st = JFO_OK;
    for (int which = 0; which < 2 && !st; ++which)
        for (int d = 0; d < 3 && !st; ++d) {
            int n = 0;
            for (int cell = 0; cell < ncells; ++cell) {
                if (is_nearby(c, cell, 0)) continue;
                double r = which == 0 ? c->bound_upper[cell * 3 + d] : c->bound_lower[cell * 3 + d];
                if (isnan(r)) st = JFO_BAD_CONFIG;  /* a far cell without a bound */
                items[n] = cell;
                rates[n] = r > 0.0 ? r : 0.0;
                ++n;
            }
            if (!st) st = walker_build(&c->walker[which][d], items, rates, n);
            if (!st && which == 1 && d == 2) c->have_walker = 1;
        }
    free(items);
    free(rates);
    return st;
}

JfoWater *jfo_water_cells_create(const JfoWaterSystem *system, int cells_per_side, int neighbor_layers,
                                 const double *positions, const double *charges, const double *roots,
                                 const double *bounds_upper, const double *bounds_lower, int keep_pairs, int far,
                                 double dipole_charge, int *status) {
    JfoWater *w = jfo_water_create(system, positions, charges, status);
    if (!w) return NULL;
    JfoSystem cs;
    memset(&cs, 0, sizeof(cs));
    cs.n = system->molecules;
    cs.system_length = system->system_length;
    cs.cells_per_side = cells_per_side;
    cs.neighbor_layers = neighbor_layers;
    cs.max_occupants = 1;
    cs.beta = system->beta;
    cs.chain_time = system->chain_time;
    cs.speed = system->speed;
    cs.initial_direction = system->initial_direction;
    cs.initial_active = system->initial_active / 3;
    cs.potential = JFO_POT_HARD_SPHERE;
    cs.far = JFO_FAR_NONE;
    cs.rng_key = system->rng_key;
    if (cells_per_side < 1 || neighbor_layers < 0 || (far != JFO_FAR_CELL_VETO && far != JFO_FAR_CELL_BOUNDING)) {
        jfo_water_destroy(w);
        *status = JFO_BAD_CONFIG;
        return NULL;
    }
    /* the occupancy takes the root units in the order of the root nodes (initialize, :95-121) */
    w->cells = jfo_chain_create(&cs, roots, NULL, status);
    if (!w->cells) {
        jfo_water_destroy(w);
        return NULL;
    }
    *status = chain_install_bounds(w->cells, bounds_upper, bounds_lower);
    if (*status) {
        jfo_water_destroy(w);
        return NULL;
    }
    w->root_speed = system->speed * (1.0 / 3.0);
    w->keep_pairs = keep_pairs ? 1 : 0;
    w->far = far;
    w->dipole_charge = dipole_charge;
    w->pairs_valid = 0;
    return w;
}

/* x_d <- (x_d + v_d (t - t_stamp)) % L along the direction of motion (the other components add 0.0) */
static void water_slice(const JfoWater *w, double *p, double speed, double q, double r, double from_q, double from_r) {
    double dt = jfo_time_sub(q, r, from_q, from_r);
    for (int d = 0; d < 3; ++d) {
        double v = d == w->direction ? speed : 0.0;
        p[d] = jfo_py_mod(p[d] + v * dt, w->sys.system_length);
    }
}

static int64_t water_cells_run(JfoWater *w, int64_t max_events, JfoEvent *log, double *root_log, int *status) {
    const JfoWaterSystem *s = &w->sys;
    JfoChain *c = w->cells;
    const int M = s->molecules;
    int64_t done = 0;
    *status = JFO_OK;
    while (done < max_events) {
        const int a = w->active, m = a / 3, t = a % 3;
        double *root = &c->pos[3 * m];
        double velocity[3] = {0.0, 0.0, 0.0};
        velocity[w->direction] = s->speed;
        c->active = m;
        c->direction = w->direction;
        int st = occ_update(c);
        if (st) {
            *status = st;
            return done;
        }
        Cand best;
        best.q = INFINITY;
        best.r = INFINITY;
        best.kind = 1 << 30;
        best.target = 1 << 30;
        best.aux = -1;
        best.rate = 0.0;
        if (!w->pairs_valid) {
            /* the bonds of the active unit's molecule and Lennard-Jones between oxygens (the factor-type-map taggers),
             * created with the event: their in-state copies are the current active leaf and root unit */
            Cand pair = best;
            for (int u = 0; u < 3 && !st; ++u) {
                if (u == t) continue;
                const MH *bond = (t == 1 || u == 1) ? &w->oh : &w->hh;
                int b = 3 * m + u;
                double sep[3], dt;
                water_separation(w, a, b, sep);
                double du = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_PAIR, b), s->beta);
                st = mh_displacement(bond, velocity, sep, du, &dt);
                if (!st) offer(&pair, w->ts_q, w->ts_r, dt, JFO_EV_BOND, b, -1, 0.0);
            }
            for (int other = 0; other < M && !st && t == 1; ++other) {
                if (other == m) continue;
                int b = 3 * other + 1;
                double sep[3], dt;
                water_separation(w, a, b, sep);
                double du = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_PAIR, b), s->beta);
                st = mh_displacement(&w->lj, velocity, sep, du, &dt);
                if (!st) offer(&pair, w->ts_q, w->ts_r, dt, JFO_EV_PAIR, b, -1, 0.0);
            }
            if (st) {
                *status = st;
                return done;
            }
            w->pair = pair;
            w->pairs_valid = 1;
            memcpy(w->snap_leaf, &w->pos[3 * a], sizeof(w->snap_leaf));
            memcpy(w->snap_root, root, sizeof(w->snap_root));
            w->snap_q = w->ts_q;
            w->snap_r = w->ts_r;
        }
        if (cand_better(&w->pair, &best)) best = w->pair;
        /* the summed-bounding Coulomb factor with the occupants of the nearby cells, then the surplus molecules */
        int ax[3];
        cell_axes(c, c->occ_cell, ax);
        int n_off = 0, offsets[64];
        for (int o = 0; o < c->m; ++o)
            if (c->near_axis[o]) offsets[n_off++] = o;
        for (int pass = 0; pass < 2 && !st; ++pass) {
            int first = 0, last = pass == 0 ? n_off * n_off * n_off : c->ncells;
            for (int k = first; k < last && !st; ++k) {
                int cell, count, *list;
                if (pass == 0) {
                    int ox = k % n_off, oy = (k / n_off) % n_off, oz = k / (n_off * n_off);
                    cell = (ax[0] + offsets[ox]) % c->m + c->m * ((ax[1] + offsets[oy]) % c->m) +
                           c->m * c->m * ((ax[2] + offsets[oz]) % c->m);
                    count = c->occ_count[cell];
                    list = &c->occ[cell * c->cap];
                } else {
                    cell = k;
                    count = c->sur_count[cell];
                    list = &c->sur[(size_t)cell * c->sys.n];
                }
                for (int i = 0; i < count && !st; ++i) {
                    int other = list[i];
                    double du[3], dt;
                    for (int j = 0; j < 3; ++j)
                        du[j] = jfo_expovariate(
                            jfo_draw(s->rng_key, w->event, JFO_RNG_COMPOSITE, (uint32_t)(3 * other + j)), s->beta);
                    st = jfo_composite_event_time(3, s->ewald_alpha, s->fourier_cutoff, s->position_cutoff,
                                                  s->coulomb_prefactor, s->bound_prefactor, s->system_length,
                                                  velocity, &w->pos[3 * a], w->charge[a], &w->pos[9 * other],
                                                  &w->charge[3 * other], du, &dt);
                    if (!st) offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_COMPOSITE, other, -1, 0.0);
                }
            }
        }
        if (st) {
            *status = st;
            return done;
        }
        int active_cell;
        st = cell_of(c, root, &active_cell);
        if (st) {
            *status = st;
            return done;
        }
        if (w->far == JFO_FAR_CELL_BOUNDING) {
            /* CellBoundingPotentialTagger (cell_bounding_potential_tagger.py:127-155): the occupant of every occupied
             * cell that is not nearby; TwoCompositeObjectCellBoundingPotentialEventHandler.send_event_time
             * (two_composite_object_cell_bounding_potential_event_handler.py:153-207): the relative cell of the target's
             * root cell to the active root's, the bound of that cell times the charge factor
             * (CellBoundingPotential.standard_velocity_displacement, cell_bounding_potential.py:155-198) */
            for (int cell = 0; cell < c->ncells && !st; ++cell) {
                if (c->occ_count[cell] == 0 || is_nearby(c, cell, active_cell)) continue;
                int other = c->occ[cell * c->cap], target_cell;
                st = cell_of(c, &c->pos[3 * other], &target_cell);
                if (st) break;
                int rc = relative_cell(c, target_cell, active_cell);
                if (is_nearby(c, rc, 0)) {
                    st = JFO_ASSERT;
                    break;
                }
                double lower[3], rate, dt;
                for (int d = 0; d < 3; ++d) lower[d] = -c->bound_lower[rc * 3 + d];
                double du = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_CELL_BOUND, (uint32_t)other), s->beta);
                st = jfo_composite_cell_bound_time(&c->bound_upper[rc * 3], lower, velocity, w->charge[a],
                                                   &w->charge[3 * other], 3, w->dipole_charge, du, &rate, &dt);
                if (!st) offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_CELL_BOUNDING, other, active_cell, rate);
            }
            if (st) {
                *status = st;
                return done;
            }
        } else {
            /* the molecular cell veto: the charge factor is the active unit's charge
             * (DipoleMonteCarloEstimator.charge_correction_factor without target charges) */
            double charge_factor = w->charge[a];
            int which = 0;
            if (!(charge_factor > 0.0)) {
                charge_factor *= -1.0;
                which = 1;
            }
            const Walker *wk = &c->walker[which][w->direction];
            double total_rate = wk->total_rate * charge_factor;
            int rc = walker_sample(wk, jfo_draw(s->rng_key, w->event, JFO_RNG_VETO_CHOICE, 0),
                                   jfo_draw(s->rng_key, w->event, JFO_RNG_VETO_UNIFORM, 0));
            double rate = (which == 0 ? c->bound_upper[rc * 3 + w->direction] : c->bound_lower[rc * 3 + w->direction]) *
                          charge_factor;
            if (!(rate > 0.0)) {
                *status = JFO_ASSERT;
                return done;
            }
            int target_cell = translate_cell(c, active_cell, rc);
            double dt = jfo_expovariate(jfo_draw(s->rng_key, w->event, JFO_RNG_VETO_TIME, 0), s->beta) /
                        (total_rate * s->speed);
            offer(&best, w->ts_q, w->ts_r, dt, JFO_EV_CELL_VETO, -1, target_cell, rate);
        }
        {
            /* the cell boundary of the active root unit */
            int cax[3];
            cell_axes(c, active_cell, cax);
            int d = w->direction;
            double boundary = c->cmin[(cax[d] + 1) % c->m];
            double sep = boundary - root[d];
            if (sep < 0.0) sep = sep + s->system_length;
            offer(&best, w->ts_q, w->ts_r, sep / w->root_speed, JFO_EV_BOUNDARY, -1, -1, boundary);
        }
        {
            Cand e;
            e.q = w->eoc_q;
            e.r = w->eoc_r;
            e.kind = JFO_EV_END_OF_CHAIN;
            e.target = w->eoc_new_active;
            e.aux = -1;
            e.rate = 0.0;
            if (cand_better(&e, &best)) best = e;
        }
        /* commit: the active leaf and root unit time-sliced to the event time, from the in-state of the winner */
        JfoEvent ev;
        ev.kind = best.kind;
        ev.moved = a;
        ev.target = best.target;
        ev.accepted = 1;
        ev.time_q = best.q;
        ev.time_r = best.r;
        if (best.kind == JFO_EV_BOND || best.kind == JFO_EV_PAIR) {
            memcpy(&w->pos[3 * a], w->snap_leaf, sizeof(w->snap_leaf));
            memcpy(root, w->snap_root, sizeof(w->snap_root));
            water_slice(w, &w->pos[3 * a], s->speed, best.q, best.r, w->snap_q, w->snap_r);
            water_slice(w, root, w->root_speed, best.q, best.r, w->snap_q, w->snap_r);
        } else {
            water_slice(w, &w->pos[3 * a], s->speed, best.q, best.r, w->ts_q, w->ts_r);
            water_slice(w, root, w->root_speed, best.q, best.r, w->ts_q, w->ts_r);
        }
        w->ts_q = best.q;
        w->ts_r = best.r;
        switch (best.kind) {
        case JFO_EV_BOND:
        case JFO_EV_PAIR:
            w->active = best.target;
            break;
        case JFO_EV_COMPOSITE:
        case JFO_EV_CELL_BOUNDING:
        case JFO_EV_CELL_VETO: {
            int other = best.target;
            if (best.kind == JFO_EV_CELL_BOUNDING) {
                /* send_out_state (:209-265): the active root must still be in the cell of the event time's
                 * candidate (the reference returns no out-state otherwise, which its mediator cannot insert); the
                 * thinning draws against the bounding event rate times the speed */
                int now_cell;
                st = cell_of(c, root, &now_cell);
                if (st || now_cell != best.aux) {
                    *status = st ? st : JFO_ASSERT;
                    return done;
                }
                best.rate *= s->speed;
            }
            if (best.kind == JFO_EV_CELL_VETO) {
                /* the occupant of the sampled cell, looked up at the commit (Mediator.get_arguments_cell_veto_event_handler) */
                other = c->occ_count[best.aux] > 0 ? c->occ[best.aux * c->cap] : -1;
                ev.target = other;
                ev.accepted = 0;
                if (other < 0) break;
            }
            int new_active;
            double draws[3], bounding, rate;
            draws[0] = jfo_uniform(jfo_draw(s->rng_key, w->event, JFO_RNG_THIN, 0));
            draws[1] = jfo_uniform(jfo_draw(s->rng_key, w->event, JFO_RNG_LIFT, 0));
            draws[2] = draws[1];
            if (best.kind == JFO_EV_COMPOSITE)
                st = jfo_composite_out_state(3, s->lifting, 1, s->ewald_alpha, s->fourier_cutoff, s->position_cutoff,
                                             s->coulomb_prefactor, s->bound_prefactor, s->system_length, velocity,
                                             &w->pos[9 * m], &w->charge[3 * m], t, &w->pos[9 * other],
                                             &w->charge[3 * other], m < other, draws, &new_active, &bounding, &rate);
            else
                st = jfo_composite_bounded_out_state(3, s->lifting, 1, s->ewald_alpha, s->fourier_cutoff,
                                                     s->position_cutoff, s->coulomb_prefactor, s->system_length,
                                                     velocity, &w->pos[9 * m], &w->charge[3 * m], t,
                                                     &w->pos[9 * other], &w->charge[3 * other], m < other, best.rate,
                                                     draws, &new_active, &rate);
            if (st) {
                *status = st;
                return done;
            }
            ev.accepted = new_active >= 0;
            if (new_active >= 0) w->active = new_active < 3 ? 3 * m + new_active : 3 * other + (new_active - 3);
            break;
        }
        case JFO_EV_BOUNDARY:
            root[w->direction] = best.rate;
            ev.accepted = 0;
            break;
        case JFO_EV_END_OF_CHAIN:
            w->direction = (w->direction + 1) % 3;
            w->active = best.target;
            jfo_time_add(w->ts_q, w->ts_r, jfo_time_sub(w->ts_q, w->ts_r, w->ts_q, w->ts_r) + s->chain_time,
                         &w->eoc_q, &w->eoc_r);
            w->eoc_new_active = water_new_active(w, (uint64_t)(w->event + 1));
            break;
        default:
            *status = JFO_ASSERT;
            return done;
        }
        /* every event but the cell boundary trashes the bond and Lennard-Jones candidates */
        if (best.kind != JFO_EV_BOUNDARY || !w->keep_pairs) w->pairs_valid = 0;
        ev.new_active = w->active;
        ev.new_direction = w->direction;
        ev.x = w->pos[3 * a];
        ev.y = w->pos[3 * a + 1];
        ev.z = w->pos[3 * a + 2];
        if (log) log[done] = ev;
        if (root_log) memcpy(&root_log[3 * done], root, sizeof(double) * 3);
        w->event++;
        done++;
    }
    return done;
}

void jfo_water_roots(const JfoWater *w, double *roots) {
    if (w->cells) memcpy(roots, w->cells->pos, sizeof(double) * 3 * (size_t)w->sys.molecules);
}

void jfo_water_positions(const JfoWater *w, double *positions) {
    memcpy(positions, w->pos, sizeof(double) * 3 * (size_t)w->units);
}

void jfo_water_state(const JfoWater *w, int64_t *event_count, int *active, int *direction, double *time_q,
                     double *time_r) {
    *event_count = w->event;
    *active = w->active;
    *direction = w->direction;
    *time_q = w->ts_q;
    *time_r = w->ts_r;
}
