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
};

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
__device__ inline int composite_out_state(const CompositeModel &m, int draw_mode, const double *velocity,
                                          const double *locals, const double *local_charges, int active,
                                          const double *targets, const double *target_charges, int local_first,
                                          const double *draws, int &new_active, double &bounding_rate,
                                          double &event_rate) {
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
        bound[j] = bound_derivative(m, d, speed, s, ca, target_charges[j]);
        pair[j] = coulomb_derivative(m, d, speed, s, ca, target_charges[j]);
    }
    if (!composite_thinning(m, draw_mode, bound, pair, draws, target_factor, bounding_rate, event_rate))
        return JFGPU_STATUS_OK;
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

}  // namespace jf
