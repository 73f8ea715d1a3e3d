// jf_lifting.cuh -- the lifting schemes of composite objects: which unit becomes active after an event whose
// interaction involves more than two units.
//
// The table is the reference's derivative table (jellyfysh/lifting/lifting.py:47-80): the factor derivatives of the
// units in insertion order and the flag of the active unit.  Positive derivatives inserted before the active unit
// add up to a position, the active unit adds a uniform draw of [0, its derivative); the negative derivatives, negated,
// form the sequence that is searched:
//   inside-first  (inside_first_lifting.py:37-54)  the first unit whose running sum of the sequence reaches the
//                                                  position (<=), else the last;
//   outside-first (outside_first_lifting.py:38-55) the same with the position reflected, sum(sequence) - position;
//   ratio         (ratio_lifting.py:38-56)         the same with a fresh uniform draw of [0, sum(sequence)).
// The arithmetic is Python's: `+=` rounded per step, sum() with CPython 3.12's Neumaier compensation,
// random.uniform(a, b) = a + (b - a) * random().
#pragma once

#include <cmath>
#include <cstdint>

#include "jfgpu.h"

namespace jf {

// The decision of one table.  `draw` is either the value the reference's random.uniform returned
// (JFGPU_DRAW_VALUE) or the unit draw random() it formed that value from (JFGPU_DRAW_UNIT).  On success
// `selected` is the table index of the new active unit; `bound` is the upper end b of the random.uniform(0.0, b)
// call that decides (the active derivative for inside-first and outside-first, the sum of the sequence for ratio;
// NaN where the reference raises before the call).  Returns JFGPU_STATUS_*:
//   JFGPU_STATUS_ASSERTION  an active unit with a derivative <= 0 (lifting.py:76), or a second active unit (the
//                           tables of the reference hold one: lifting.py:33-34);
//   JFGPU_STATUS_LIFTING    no active unit (LiftingSchemeError, lifting.py:107-108);
//   JFGPU_STATUS_INDEX      no negative derivative (IndexError of identifiers[-1] on an empty list).
__host__ __device__ inline int lifting_select(int scheme, int draw_mode, const double *rates, const int32_t *active,
                                              int64_t count, double draw, int64_t &selected, double &bound) {
    selected = -1;
    bound = NAN;
    double position = 0.0;
    bool recorded = false;
    // sum() of the sequence, accumulated while the table is read (CPython 3.12: first term added to int 0, then
    // Neumaier compensation, the compensation added at the end when nonzero and finite)
    double total = 0.0, compensation = 0.0;
    int64_t negatives = 0, last = -1;
    for (int64_t i = 0; i < count; ++i) {
        const double rate = rates[i];
        if (rate > 0.0) {
            if (active[i]) {
                if (recorded) return JFGPU_STATUS_ASSERTION;
                recorded = true;
                if (scheme != JFGPU_LIFTING_RATIO) bound = rate;
                position += draw_mode == JFGPU_DRAW_UNIT ? 0.0 + (rate - 0.0) * draw : draw;
            } else if (!recorded) {
                position += rate;
            }
        } else {
            if (active[i]) return JFGPU_STATUS_ASSERTION;
            const double x = -rate;
            if (negatives == 0) {
                total = 0.0 + x;
            } else {
                const double t = total + x;
                if (fabs(total) >= fabs(x))
                    compensation += (total - t) + x;
                else
                    compensation += (x - t) + total;
                total = t;
            }
            ++negatives;
            last = i;
        }
    }
    if (!recorded) {
        bound = NAN;
        return JFGPU_STATUS_LIFTING;
    }
    if (compensation != 0.0 && isfinite(compensation)) total += compensation;
    if (scheme == JFGPU_LIFTING_OUTSIDE_FIRST) {
        position = total - position;
    } else if (scheme == JFGPU_LIFTING_RATIO) {
        bound = total;
        position = draw_mode == JFGPU_DRAW_UNIT ? 0.0 + (total - 0.0) * draw : draw;
    }
    if (negatives == 0) return JFGPU_STATUS_INDEX;
    double summed = 0.0;
    for (int64_t i = 0; i < count; ++i) {
        const double rate = rates[i];
        if (rate > 0.0) continue;
        summed += -rate;
        if (position <= summed) {
            selected = i;
            return JFGPU_STATUS_OK;
        }
    }
    selected = last;
    return JFGPU_STATUS_OK;
}

}  // namespace jf
