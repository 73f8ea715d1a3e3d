// jf_composite.cuh -- events between two composite objects (water molecules, dipoles) whose point charges interact
// by the merged-image Coulomb potential, bounded per pair by the inverse-power Coulomb bound and summed over the
// target object (TwoCompositeObjectSummedBoundingPotentialEventHandler,
// event_handler/two_composite_object_summed_bounding_potential_event_handler.py:119-202).
//
// Candidate time: the smallest bounded displacement over the target object's units, each with its own potential
// change.  Out-state at the event: thinning of the summed positive bound against the active unit's factor
// derivative, then the derivative table of both objects (event_handler_with_bounding_potential.py:170-220) and the
// lifting scheme (jf_lifting.cuh) name the new active unit.  All in FP64 with the reference's arithmetic.
#pragma once

#include "jf_device.cuh"
#include "jf_lifting.cuh"

namespace jf {

constexpr int kMaxCompositeUnits = 8;  // leaf units per composite object

struct CompositeModel {
    MIC mic;                  // merged-image Coulomb (its Fourier table on the device)
    double coulomb_prefactor; // MergedImageCoulombPotential prefactor
    double bound_prefactor;   // InversePowerCoulombBoundingPotential prefactor
    double system_length;
    int units;                // leaf units per composite object
    int lifting;              // JFGPU_LIFTING_*
    // the terms of the merged-image sum in lists, for a warp that shares one evaluation (mic_x_warp): the
    // real-space images (i, j, k) and the Fourier rows (i, j, last k) of the reference's loops
    const int4 *images = nullptr;
    const int4 *rows = nullptr;
    int n_images = 0, n_rows = 0;
    // FP32 copies of the merged-image constants and Fourier table, for the screened thinning (mic_x_warp32)
    const float *fourier32 = nullptr;
    float alpha_over_length32 = 0.f, alpha_over_length_sq32 = 0.f, two_alpha_over_length_root_pi32 = 0.f;
    float system_length32 = 0.f, two_pi_over_length32 = 0.f;
};

// mic_x_warp in FP32 with an absolute error bound, for decisions that need the sum only to within that bound.
// The bound covers the rounding of the separation to FP32 and the FP32 evaluation: an image term x (c exp(-a^2 r^2)
// + erfc(a r) / r) / r^2 within 4096 ulp of its magnitude (the argument errors of exp and erfc grow with a^2 r^2,
// at most about 75 here, times the documented 2-4 ulp of expf and erfcf), a Fourier term within 512 ulp of its
// coefficient (the recurrences of sin and cos over at most 18 steps from angles known to 2 ulp), and the additions.
static __device__ __noinline__ void mic_x_warp32(const CompositeModel &c, float sx, float sy, float sz, int lane,
                                                 float &value, float &error) {
    const int n = c.mic.fourier_cutoff + 1;
    const float length = c.system_length32;
    float derivative = 0.f, image_magnitude = 0.f, fourier_magnitude = 0.f;
    for (int e = lane; e < c.n_images; e += 32) {
        const int4 image = c.images[e];
        const float vz = sz + (float)image.z * length, vy = sy + (float)image.y * length;
        const float vector_x = sx + (float)image.x * length;
        const float vector_sq = vector_x * vector_x + vy * vy + vz * vz;
        const float vector_norm = sqrtf(vector_sq);
        const float term = vector_x *
                           (c.two_alpha_over_length_root_pi32 * expf(-c.alpha_over_length_sq32 * vector_sq) +
                            erfcf(c.alpha_over_length32 * vector_norm) / vector_norm) /
                           vector_sq;
        derivative += term;
        image_magnitude += fabsf(term);
    }
    if (c.n_rows > 0 && 31 - lane < c.n_rows) {
        float delta_sin_x, delta_cos_x, delta_sin_y, delta_cos_y, delta_sin_z, delta_cos_z;
        sincosf(c.two_pi_over_length32 * sx, &delta_sin_x, &delta_cos_x);
        sincosf(c.two_pi_over_length32 * sy, &delta_sin_y, &delta_cos_y);
        sincosf(c.two_pi_over_length32 * sz, &delta_sin_z, &delta_cos_z);
        for (int e = 31 - lane; e < c.n_rows; e += 32) {
            const int4 row = c.rows[e];
            float cos_x = delta_cos_x, sin_x = delta_sin_x, store;
            for (int i = 1; i < row.x; ++i) {
                store = cos_x;
                cos_x = store * delta_cos_x - sin_x * delta_sin_x;
                sin_x = sin_x * delta_cos_x + store * delta_sin_x;
            }
            float cos_y = 1.f, sin_y = 0.f;
            for (int j = 0; j < row.y; ++j) {
                store = cos_y;
                cos_y = store * delta_cos_y - sin_y * delta_sin_y;
                sin_y = sin_y * delta_cos_y + store * delta_sin_y;
            }
            float cos_z = 1.f, sin_z = 0.f;
            for (int k = 0; k < row.z + 1; ++k) {
                const float coefficient = c.fourier32[(row.x * n + row.y) * n + k];
                derivative += coefficient * sin_x * cos_y * cos_z;
                fourier_magnitude += fabsf(coefficient);
                store = cos_z;
                cos_z = store * delta_cos_z - sin_z * delta_sin_z;
                sin_z = sin_z * delta_cos_z + store * delta_sin_z;
            }
        }
    }
    for (int offset = 16; offset > 0; offset >>= 1) {
        derivative += __shfl_xor_sync(0xffffffffu, derivative, offset);
        image_magnitude += __shfl_xor_sync(0xffffffffu, image_magnitude, offset);
        fourier_magnitude += __shfl_xor_sync(0xffffffffu, fourier_magnitude, offset);
    }
    value = derivative;
    const float ulp = 5.9604645e-8f;  // 2^-24
    error = ulp * (4096.f * image_magnitude + 512.f * fourier_magnitude) + fabsf(derivative) * (16.f * ulp);
}

// The x-derivative of the merged-image sum (mic_x) shared by the 32 lanes of a warp: lane l takes the real-space
// images l, l + 32, ... and the Fourier rows (i, j) 31 - l, 63 - l, ...; each term is computed with the reference's
// arithmetic (the cos/sin recurrences rebuilt up to the lane's row), so every term equals mic_x's, and the lanes'
// sums are added by a butterfly that leaves the same total in every lane.  Only the order of the additions differs
// from mic_x's (a rounding of the sum, about 1e-16 relative).  Every lane of the warp must call it with the same
// separation.
static __device__ __noinline__ double mic_x_warp(const CompositeModel &c, double sx, double sy, double sz, int lane) {
    const MIC &m = c.mic;
    const int n = m.fourier_cutoff + 1;
    double derivative = 0.0;
    for (int e = lane; e < c.n_images; e += 32) {
        const int4 image = c.images[e];
        const double vector_z_sq = (sz + image.z * m.system_length) * (sz + image.z * m.system_length);
        const double vector_y_sq = (sy + image.y * m.system_length) * (sy + image.y * m.system_length);
        const double vector_x = sx + image.x * m.system_length;
        const double vector_sq = vector_x * vector_x + vector_y_sq + vector_z_sq;
        const double vector_norm = sqrt(vector_sq);
        derivative += vector_x *
                      (m.two_alpha_over_length_root_pi * exp(-m.alpha_over_length_sq * vector_sq) +
                       erfc(m.alpha_over_length * vector_norm) / vector_norm) /
                      vector_sq;
    }
    if (c.n_rows > 0 && 31 - lane < c.n_rows) {
        const double delta_cos_x = cos(m.two_pi_over_length * sx);
        const double delta_sin_x = sin(m.two_pi_over_length * sx);
        const double delta_cos_y = cos(m.two_pi_over_length * sy);
        const double delta_sin_y = sin(m.two_pi_over_length * sy);
        const double delta_cos_z = cos(m.two_pi_over_length * sz);
        const double delta_sin_z = sin(m.two_pi_over_length * sz);
        for (int e = 31 - lane; e < c.n_rows; e += 32) {
            const int4 row = c.rows[e];  // (i, j, last k, unused)
            double cos_x = delta_cos_x, sin_x = delta_sin_x, store;
            for (int i = 1; i < row.x; ++i) {
                store = cos_x;
                cos_x = store * delta_cos_x - sin_x * delta_sin_x;
                sin_x = sin_x * delta_cos_x + store * delta_sin_x;
            }
            double cos_y = 1.0, sin_y = 0.0;
            for (int j = 0; j < row.y; ++j) {
                store = cos_y;
                cos_y = store * delta_cos_y - sin_y * delta_sin_y;
                sin_y = sin_y * delta_cos_y + store * delta_sin_y;
            }
            double cos_z = 1.0, sin_z = 0.0;
            for (int k = 0; k < row.z + 1; ++k) {
                derivative += m.fourier[(row.x * n + row.y) * n + k] * sin_x * cos_y * cos_z;
                store = cos_z;
                cos_z = store * delta_cos_z - sin_z * delta_sin_z;
                sin_z = sin_z * delta_cos_z + store * delta_sin_z;
            }
        }
    }
    for (int offset = 16; offset > 0; offset >>= 1) derivative += __shfl_xor_sync(0xffffffffu, derivative, offset);
    return derivative;
}

// mic_x_warp over a group of GW lanes (8 or 16) of a warp in which several chains each have a group: every lane takes
// the terms of 32 / GW of mic_x_warp's lanes (lane l, l + GW, ...) into separate partial sums, and the partial sums
// are combined in the order of mic_x_warp's butterfly (offsets 16, 8, ... 1; the offsets of at least GW between a
// lane's own partial sums, the smaller ones by shuffles within the group), so that the value equals mic_x_warp's bit
// for bit.  mask: the lanes of every group that calls it (whole groups).
template <int GW>
__device__ inline double mic_x_group(const CompositeModel &c, double sx, double sy, double sz, int glane,
                                     unsigned mask) {
    constexpr int V = 32 / GW;
    const MIC &m = c.mic;
    const int n = m.fourier_cutoff + 1;
    double part[V];
#pragma unroll
    for (int k = 0; k < V; ++k) part[k] = 0.0;
#pragma unroll
    for (int k = 0; k < V; ++k) {
        const int lane = glane + GW * k;
        double derivative = 0.0;
        for (int e = lane; e < c.n_images; e += 32) {
            const int4 image = c.images[e];
            const double vector_z_sq = (sz + image.z * m.system_length) * (sz + image.z * m.system_length);
            const double vector_y_sq = (sy + image.y * m.system_length) * (sy + image.y * m.system_length);
            const double vector_x = sx + image.x * m.system_length;
            const double vector_sq = vector_x * vector_x + vector_y_sq + vector_z_sq;
            const double vector_norm = sqrt(vector_sq);
            derivative += vector_x *
                          (m.two_alpha_over_length_root_pi * exp(-m.alpha_over_length_sq * vector_sq) +
                           erfc(m.alpha_over_length * vector_norm) / vector_norm) /
                          vector_sq;
        }
        if (c.n_rows > 0 && 31 - lane < c.n_rows) {
            const double delta_cos_x = cos(m.two_pi_over_length * sx);
            const double delta_sin_x = sin(m.two_pi_over_length * sx);
            const double delta_cos_y = cos(m.two_pi_over_length * sy);
            const double delta_sin_y = sin(m.two_pi_over_length * sy);
            const double delta_cos_z = cos(m.two_pi_over_length * sz);
            const double delta_sin_z = sin(m.two_pi_over_length * sz);
            for (int e = 31 - lane; e < c.n_rows; e += 32) {
                const int4 row = c.rows[e];
                double cos_x = delta_cos_x, sin_x = delta_sin_x, store;
                for (int i = 1; i < row.x; ++i) {
                    store = cos_x;
                    cos_x = store * delta_cos_x - sin_x * delta_sin_x;
                    sin_x = sin_x * delta_cos_x + store * delta_sin_x;
                }
                double cos_y = 1.0, sin_y = 0.0;
                for (int j = 0; j < row.y; ++j) {
                    store = cos_y;
                    cos_y = store * delta_cos_y - sin_y * delta_sin_y;
                    sin_y = sin_y * delta_cos_y + store * delta_sin_y;
                }
                double cos_z = 1.0, sin_z = 0.0;
                for (int kk = 0; kk < row.z + 1; ++kk) {
                    derivative += m.fourier[(row.x * n + row.y) * n + kk] * sin_x * cos_y * cos_z;
                    store = cos_z;
                    cos_z = store * delta_cos_z - sin_z * delta_sin_z;
                    sin_z = sin_z * delta_cos_z + store * delta_sin_z;
                }
            }
        }
        part[k] = derivative;
    }
    // the butterfly: lane v adds lane v ^ offset; v = glane + GW k, so an offset of at least GW pairs k with k ^ step
#pragma unroll
    for (int offset = 16; offset >= GW; offset >>= 1) {
        const int step = offset / GW;
        double next[V];
#pragma unroll
        for (int k = 0; k < V; ++k) next[k] = part[k] + part[k ^ step];
#pragma unroll
        for (int k = 0; k < V; ++k) part[k] = next[k];
    }
    double derivative = part[0];
#pragma unroll
    for (int offset = GW / 2; offset > 0; offset >>= 1) derivative += __shfl_xor_sync(mask, derivative, offset);
    return derivative;
}

// HypercubicPeriodicBoundaries.separation_vector (setting/hypercubic_setting.py:120-140, :156-172)
__device__ inline void periodic_separation(const double *from, const double *to, double length, double *s) {
    const double half = length / 2.0;
    for (int d = 0; d < 3; ++d) s[d] = py_mod_near((to[d] - from[d]) + half, length) - half;
}

// InversePowerCoulombBoundingPotential.derivative (potential.py:187-219 with the C extension's x-derivative)
__device__ inline double bound_derivative(const CompositeModel &m, int d, double speed, const double *s, double c1,
                                          double c2) {
    double p[3];
    permute3(s, d, p);
    return ipcb_x_derivative(m.bound_prefactor * c1 * c2, p[0], p[1], p[2]) * speed;
}

// MergedImageCoulombPotential.derivative (potential.py:187-219, merged_image_coulomb_potential.py:128-154)
__device__ inline double coulomb_derivative(const CompositeModel &m, int d, double speed, const double *s, double c1,
                                            double c2) {
    return mic_std_derivative(m.mic, m.coulomb_prefactor, d, s, c1, c2) * speed;
}

// coulomb_derivative with the merged-image sum shared by the warp (mic_x_warp); every lane gets the value
__device__ inline double coulomb_derivative_warp(const CompositeModel &m, int d, double speed, const double *s,
                                                 double c1, double c2, int lane) {
    double p[3];
    permute3(s, d, p);
    return m.coulomb_prefactor * c1 * c2 * mic_x_warp(m, p[0], p[1], p[2], lane) * speed;
}

// ipcb_x_displacement in FP32, to screen candidates: the same steps (inverse_power_coulomb_bounding_potential.c:
// 85-139) on FP32 inputs, with a first-order bound `error` on the absolute difference from the exact value.  Each
// step's relative error is counted in units of 2^-24 (inputs rounded from FP64, correctly rounded +, -, *, / and
// sqrtf) and carried through the differences and the square root; du_error is the bound on du.  `unsafe` is set
// where the first-order bound does not hold or the case is rare enough to leave to FP64: a whole box or more of
// potential change, a branch decided within the bounds, a radicand within four bounds of zero, a non-finite value.
__device__ inline float ipcb_x_displacement32(float pp, float sx, float sy, float sz, float du, float du_error,
                                              float length, float &error, bool &unsafe) {
    const float u = 0x1p-24f;
    const float half = 0.5f * length;
    const float perp = sy * sy + sz * sz;                           // 4u
    float current = pp / sqrtf(sx * sx + perp);                     // 8u
    const float u_zero = pp / sqrtf(perp);                          // 7u
    const float u_half = pp / sqrtf(half * half + perp);            // 8u
    const float per_length = fabsf(u_zero - u_half);
    if (!(du < 0.9f * per_length)) unsafe = true;                   // whole boxes of potential change
    float current_error = 8.f * u * fabsf(current);
    float shift = 0.f, shift_error = 0.f;  // displacement before the final solve
    float x = sx, x_error = u * fabsf(sx);
    float sign = pp > 0.f ? -1.f : 1.f;     // displacement += x -/+ sqrt(...)
    if (pp > 0.f) {
        if (sx <= 0.f) {
            shift = half + sx;
            shift_error = u * (half + fabsf(sx)) + u * fabsf(shift);
            x = half;
            x_error = 0.f;
            current = u_half;
            current_error = 8.f * u * fabsf(u_half);
        } else {
            const float rise = u_zero - current;
            const float rise_error = 7.f * u * fabsf(u_zero) + current_error + u * fabsf(rise);
            if (fabsf(du - rise) <= 2.f * (rise_error + du_error)) unsafe = true;
            if (du >= rise) {
                du = du - rise;
                du_error += rise_error + u * fabsf(du);
                shift = sx + half;
                shift_error = u * fabsf(sx) + u * fabsf(shift);
                x = half;
                x_error = 0.f;
                current = u_half;
                current_error = 8.f * u * fabsf(u_half);
            }
        }
    } else {
        if (sx > 0.f) {
            shift = sx;
            shift_error = u * fabsf(sx);
            x = 0.f;
            x_error = 0.f;
            current = u_zero;
            current_error = 7.f * u * fabsf(u_zero);
        } else {
            const float rise = u_half - current;
            const float rise_error = 8.f * u * fabsf(u_half) + current_error + u * fabsf(rise);
            if (fabsf(du - rise) <= 2.f * (rise_error + du_error)) unsafe = true;
            if (du >= rise) {
                du = du - rise;
                du_error += rise_error + u * fabsf(du);
                shift = sx + length;
                shift_error = u * fabsf(sx) + u * fabsf(shift);
                x = 0.f;
                x_error = 0.f;
                current = u_zero;
                current_error = 7.f * u * fabsf(u_zero);
            }
        }
    }
    const float denominator = current + du;
    const float denominator_error = current_error + du_error + u * fabsf(denominator);
    if (!(fabsf(denominator) > 4.f * denominator_error)) unsafe = true;
    const float new_norm = pp / denominator;
    const float new_norm_relative = denominator_error / fabsf(denominator) + 2.f * u;
    const float radicand = new_norm * new_norm - perp;
    const float radicand_error = (2.f * new_norm_relative + u) * new_norm * new_norm + 4.f * u * perp +
                                 u * fabsf(radicand);
    if (!(radicand > 4.f * radicand_error)) unsafe = true;
    const float root = sqrtf(fmaxf(radicand, 0.f));
    const float root_error = radicand_error / (2.f * fmaxf(root, 1e-30f)) + u * root;
    const float tail = x + sign * root;
    const float value = shift + tail;
    error = 2.f * (shift_error + x_error + root_error + u * fabsf(tail) + u * fabsf(value)) + u * length;
    if (!isfinite(value) || !isfinite(error)) unsafe = true;
    return value;
}

// send_event_time (:119-150): min over the target units of the bounding displacement (Python's min keeps the first
// of equal values).  targets [units][3], target_charges [units], potential_changes [units].
__device__ inline int composite_event_time(const CompositeModel &m, const double *velocity, const double *active,
                                           double active_charge, const double *targets, const double *target_charges,
                                           const double *potential_changes, double &displacement) {
    int d;
    double speed;
    JF_TRY(analyse_velocity(velocity, d, speed));
    for (int j = 0; j < m.units; ++j) {
        double s[3], p[3];
        periodic_separation(active, targets + 3 * j, m.system_length, s);
        permute3(s, d, p);
        const double value = ipcb_x_displacement(m.bound_prefactor * active_charge * target_charges[j], p[0], p[1],
                                                 p[2], potential_changes[j], m.system_length) / speed;
        if (j == 0 || value < displacement) displacement = value;
    }
    return JFGPU_STATUS_OK;
}

// The thinning of send_out_state (:171-192) from the pair derivatives of the active unit against the target units
// (bound[j]: bounding potential, pair[j]: potential), in the reference's order of additions.  Fills target_factor
// (0.0 - pair[j], the start of _fill_lifting's target derivatives) and returns whether the event is confirmed.
__device__ inline bool composite_thinning(const CompositeModel &m, int draw_mode, const double *bound,
                                          const double *pair, const double *draws, double *target_factor,
                                          double &bounding_rate, double &event_rate) {
    bounding_rate = 0.0;
    double factor = 0.0;
    for (int j = 0; j < m.units; ++j) {
        bounding_rate += bound[j] > 0.0 ? bound[j] : 0.0;  // max(0.0, b)
        factor += pair[j];
        target_factor[j] = 0.0 - pair[j];
    }
    event_rate = factor > 0.0 ? factor : 0.0;
    const double thinning = draw_mode == JFGPU_DRAW_UNIT ? 0.0 + (bounding_rate - 0.0) * draws[0] : draws[0];
    return !(event_rate <= thinning);
}

// The thinning against a given bounding event rate (the molecular cell-bounding handler,
// two_composite_object_cell_bounding_potential_event_handler.py:231-253, and the molecular cell veto with a target,
// composite_object_cell_veto_event_handler.py:131-153): the summed pair derivatives, event_rate = max(0, sum), and
// event_rate <= uniform(0, given) rejects.  Fills target_factor as composite_thinning does.
__device__ inline int composite_given_thinning(const CompositeModel &m, int draw_mode, double given,
                                               const double *pair, const double *draws, double *target_factor,
                                               double &bounding_rate, double &event_rate, bool &confirmed) {
    // assert bounding_event_rate >= 0.0 (:243, composite_object_cell_veto_event_handler.py:150)
    if (!(given >= 0.0)) return JFGPU_STATUS_ASSERTION;
    double factor = 0.0;
    for (int j = 0; j < m.units; ++j) {
        factor += pair[j];
        target_factor[j] = 0.0 - pair[j];
    }
    bounding_rate = given;
    event_rate = factor > 0.0 ? factor : 0.0;
    const double thinning = draw_mode == JFGPU_DRAW_UNIT ? 0.0 + (bounding_rate - 0.0) * draws[0] : draws[0];
    confirmed = !(event_rate <= thinning);
    return JFGPU_STATUS_OK;
}

// _fill_lifting (event_handler_with_bounding_potential.py:170-220) and the lifting scheme, from the potential
// derivatives cross[i * units + j] of the non-active local units i against the target units j (the active
// unit's velocity).  new_active as in composite_out_state.
__device__ inline int composite_lifting(const CompositeModel &m, int draw_mode, int active, int local_first,
                                        double event_rate, double *target_factor, const double *cross,
                                        const double *draws, int &new_active) {
    const int k = m.units;
    double local_factor[kMaxCompositeUnits];
    for (int i = 0; i < k; ++i) {
        local_factor[i] = 0.0;
        if (i == active) {
            local_factor[i] = event_rate;
            continue;
        }
        for (int j = 0; j < k; ++j) {
            local_factor[i] += cross[i * k + j];
            target_factor[j] -= cross[i * k + j];
        }
    }
    double rates[2 * kMaxCompositeUnits];
    int32_t flags[2 * kMaxCompositeUnits];
    const int local_offset = local_first ? 0 : k, target_offset = local_first ? k : 0;
    for (int i = 0; i < k; ++i) {
        rates[local_offset + i] = local_factor[i];
        flags[local_offset + i] = i == active;
        rates[target_offset + i] = target_factor[i];
        flags[target_offset + i] = 0;
    }
    int64_t selected;
    double bound;
    const double draw = m.lifting == JFGPU_LIFTING_RATIO ? draws[2] : draws[1];
    const int st = lifting_select(m.lifting, draw_mode, rates, flags, 2 * k, draw, selected, bound);
    if (st != JFGPU_STATUS_OK) return st;
    const int index = (int)selected;
    new_active = index >= local_offset && index < local_offset + k ? index - local_offset : k + (index - target_offset);
    return JFGPU_STATUS_OK;
}

// send_out_state (:152-202).  locals / targets [units][3] and their charges, sorted by identifier; active is the
// index of the active unit among the locals; local_first tells whether the local object's identifier is the
// smaller one (the order of the derivative table).  draws: [0] thinning random.uniform(0.0, bounding rate),
// [1] the active unit's insert into the lifting table, [2] the ratio scheme's draw; values or unit draws as in
// lifting_select.  new_active: -1 when thinned, else 0..units-1 (a local unit) or units..2 units-1 (a target).
// given: nullptr for this handler's summed inverse-power bound; else the bounding event rate that the molecular
// cell-bounding handler (two_composite_object_cell_bounding_potential_event_handler.py:231-265) or the molecular cell
// veto with a target (composite_object_cell_veto_event_handler.py:131-162) draws the thinning against, with the same
// summed merged-image derivative, _fill_lifting and lifting after it.
__device__ inline int composite_out_state(const CompositeModel &m, int draw_mode, const double *velocity,
                                          const double *locals, const double *local_charges, int active,
                                          const double *targets, const double *target_charges, int local_first,
                                          const double *draws, int &new_active, double &bounding_rate,
                                          double &event_rate, const double *given = nullptr) {
    new_active = -1;
    bounding_rate = 0.0;
    event_rate = 0.0;
    int d;
    double speed;
    JF_TRY(analyse_velocity(velocity, d, speed));
    const int k = m.units;
    const double *a = locals + 3 * active;
    const double ca = local_charges[active];
    double bound[kMaxCompositeUnits], pair[kMaxCompositeUnits], target_factor[kMaxCompositeUnits];
    for (int j = 0; j < k; ++j) {
        double s[3];
        periodic_separation(a, targets + 3 * j, m.system_length, s);
        bound[j] = given ? 0.0 : bound_derivative(m, d, speed, s, ca, target_charges[j]);
        pair[j] = coulomb_derivative(m, d, speed, s, ca, target_charges[j]);
    }
    bool confirmed;
    if (given) {
        JF_TRY(composite_given_thinning(m, draw_mode, *given, pair, draws, target_factor, bounding_rate, event_rate,
                                        confirmed));
    } else {
        confirmed = composite_thinning(m, draw_mode, bound, pair, draws, target_factor, bounding_rate, event_rate);
    }
    if (!confirmed) return JFGPU_STATUS_OK;
    double cross[kMaxCompositeUnits * kMaxCompositeUnits];
    for (int i = 0; i < k; ++i) {
        if (i == active) continue;
        for (int j = 0; j < k; ++j) {
            double s[3];
            periodic_separation(locals + 3 * i, targets + 3 * j, m.system_length, s);
            cross[i * k + j] = coulomb_derivative(m, d, speed, s, local_charges[i], target_charges[j]);
        }
    }
    return composite_lifting(m, draw_mode, active, local_first, event_rate, target_factor, cross, draws,
                             new_active);
}

// CellBoundingPotential.standard_velocity_displacement (cell_bounding_potential.py:155-198) through
// Potential.displacement (potential/abstracts.py:212-245), with the charge factor of
// DipoleMonteCarloEstimator.charge_correction_factor (estimator/dipole_monte_carlo_estimator.py:157-190): the active
// charge times the largest absolute target charge over the estimator's dipole charge, the target charges summing to
// 0.0 by the builtin sum (asserted).  upper / lower: the relative cell's bounds in the three directions (NaN for a
// nearby cell, which the handler asserts against).  rate: the stored bounding event rate (per unit length; the
// out-state draws against rate times the speed); time: the time displacement.
__host__ __device__ inline int composite_cell_bound_time(const double *upper, const double *lower,
                                                         const double *velocity, double active_charge,
                                                         const double *target_charges, int units,
                                                         double dipole_charge, double potential_change,
                                                         double &rate, double &time) {
    int d = -1, count = 0;
    for (int c = 0; c < 3; ++c)
        if (velocity[c] != 0.0) {
            ++count;
            d = c;
        }
    if (count != 1 || !(velocity[d] > 0.0)) return JFGPU_STATUS_ASSERTION;
    const double speed = velocity[d];
    if (units < 1 || units > kMaxCompositeUnits) return JFGPU_STATUS_ASSERTION;
    // sum(target_charges) == 0.0 with CPython 3.12's compensated sum: 0 + q0 exactly, then Neumaier
    double sum = 0.0 + target_charges[0], compensation = 0.0;
    for (int j = 1; j < units; ++j) {
        const double x = target_charges[j], t = sum + x;
        compensation += fabs(sum) >= fabs(x) ? (sum - t) + x : (x - t) + sum;
        sum = t;
    }
    if (compensation != 0.0 && isfinite(compensation)) sum += compensation;
    if (sum != 0.0) return JFGPU_STATUS_ASSERTION;
    if (isnan(upper[d]) || isnan(lower[d])) return JFGPU_STATUS_ASSERTION;
    double largest = fabs(target_charges[0]);
    for (int j = 1; j < units; ++j)
        if (fabs(target_charges[j]) > largest) largest = fabs(target_charges[j]);
    if (dipole_charge == 0.0) return JFGPU_STATUS_ZERO_DIVISION;
    const double product = active_charge * largest / dipole_charge;
    rate = product > 0.0 ? upper[d] * product : lower[d] * product;
    const double displacement = rate > 0 ? potential_change / rate : INFINITY;
    time = displacement / speed;
    return JFGPU_STATUS_OK;
}

// CellVetoEventHandler.send_event_time (abstracts/cell_veto_event_handler.py:200-238) for a composite object, whose
// charge factor is the active charge (charge_correction_factor without target charges): positive, the upper bounds
// and their Walker table's total rate; else its negative and the lower ones.  upper / lower: the sampled relative
// cell's bounds, walker_upper / walker_lower: the Walker totals, each in the three directions.  rate: the bounding
// event rate of the out-state; time: potential_change / (total rate * speed).
__host__ __device__ inline int composite_cell_veto_time(const double *upper, const double *lower,
                                                        const double *walker_upper, const double *walker_lower,
                                                        const double *velocity, double active_charge,
                                                        double potential_change, double &rate, double &time) {
    int d = -1, count = 0;
    for (int c = 0; c < 3; ++c)
        if (velocity[c] != 0.0) {
            ++count;
            d = c;
        }
    if (count != 1 || !(velocity[d] > 0.0)) return JFGPU_STATUS_ASSERTION;
    const double speed = velocity[d];
    double factor = active_charge, total, bound;
    if (factor > 0.0) {
        total = walker_upper[d];
        bound = upper[d];
    } else {
        factor *= -1.0;
        total = walker_lower[d];
        bound = lower[d];
    }
    const double total_rate = total * factor;
    rate = bound * factor;
    if (!(rate > 0.0)) return JFGPU_STATUS_ASSERTION;
    const double denominator = total_rate * speed;
    if (denominator == 0.0) return JFGPU_STATUS_ZERO_DIVISION;
    time = potential_change / denominator;
    return JFGPU_STATUS_OK;
}

}  // namespace jf
