// jf_chains.cu -- the event loop of thousands of independent ECMC chains, one warp per chain.
//
// One loop iteration is one iteration of SingleProcessMediator.run (jellyfysh/mediator/single_process_mediator.py:
// 91-156) restricted to the event handlers of the path:
//   1. occupancy update of the active unit (single_active_cell_occupancy.py:149-203), lane 0;
//   2. candidate event times: nearby occupants and surplus units (excluded_cells_tagger.py:107-132,
//      surplus_cells_tagger.py:107-131 with two_leaf_unit_event_handler.py:98-138 or
//      two_leaf_unit_bounding_potential_event_handler.py:112-143), the far field (cell_bounding_potential_tagger.py:
//      127-155 with two_leaf_unit_cell_bounding_potential_event_handler.py:137-176, or
//      cell_veto_event_handler.py:162-238), the cell boundary (cell_boundary_event_handler.py:98-156) and the
//      persistent end-of-chain candidate;
//   3. the earliest candidate by a warp-shuffle argmin over (time quotient, time remainder, kind, target) in
//      place of the heap (heap_scheduler.py:111-212, heap.c:156-304);
//   4. the out-state: time slice of the active unit with periodic wrap (abstracts.py:82-95), lifting
//      (abstracts.py:283-321), thinning (event_handler_with_bounding_potential.py:75-101), boundary snap
//      (cell_boundary_event_handler.py:158-173) or end of chain (end_of_chain_event_handler.py:108-187).
//
// JFGPU_MODE_EXACT solves every candidate in FP64 with the reference's arithmetic.  JFGPU_MODE_MIXED screens
// every candidate in FP32 (jf_screen.cuh), keeps the four smallest FP32 times of every lane, and re-solves in FP64
// the candidates within (1 + 2^-10) t_min + margin and every flagged one; the winner and its event time are
// therefore the FP64 ones.  When a lane holds more than four candidates inside the margin the event is re-solved
// entirely in FP64 (counted in refine_fallbacks).
#include <cstring>
#include <map>

#include <cuda_runtime.h>

// The round kernels keep the FP64 solves and the event flow inline (no calls, no arrays in local memory): their
// latency is the chain of dependent FP64 operations, which calls and stack traffic lengthen.  The warp-per-chain FP64
// kernel calls the flow through out-of-line entry points (below).  JF_OUT_OF_LINE builds everything out of line.
#ifndef JF_OUT_OF_LINE
#define JF_SOLVE_INLINE
#define JF_FLOW_INLINE
#endif

#include "jf_engine.cuh"
#include "jf_composite.cuh"
#include "jf_screen.cuh"

namespace jf {

// The event-flow functions (candidate solves, single candidates, thinning, commit, occupancy update) are out of line
// by default; JF_FLOW_INLINE inlines them into their kernels.
#ifdef JF_FLOW_INLINE
#define JF_FLOW __forceinline__
#else
#define JF_FLOW __noinline__
#endif
#ifndef JF_REFINE_THREADS
#define JF_REFINE_THREADS 64   // threads per block of the FP64 re-solve kernel
#endif

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTopK = 4;

struct Cand {
    double q, r;
    int kind, target, aux;
    double rate;
};

__device__ inline Cand cand_none() {
    Cand c;
    c.q = kInf;
    c.r = kInf;
    c.kind = 1 << 30;
    c.target = 1 << 30;
    c.aux = -1;
    c.rate = 0.0;
    return c;
}

// earliest time first; equal times: lower kind, then lower target
// the earliest time; on equal times the lower kind, then the lower target.  The quotient and remainder of a
// candidate's time are non-negative (never -0.0, as Python's divmod gives) or +inf, so their IEEE bit patterns order
// as the values do: the comparison runs on integers, off GB300's scarce FP64 pipe.
__device__ inline bool cand_better(const Cand &a, const Cand &b) {
    const unsigned long long aq = (unsigned long long)__double_as_longlong(a.q);
    const unsigned long long bq = (unsigned long long)__double_as_longlong(b.q);
    if (aq != bq) return aq < bq;
    const unsigned long long ar = (unsigned long long)__double_as_longlong(a.r);
    const unsigned long long br = (unsigned long long)__double_as_longlong(b.r);
    if (ar != br) return ar < br;
    if (a.kind != b.kind) return a.kind < b.kind;
    return a.target < b.target;
}

__device__ inline void offer(Cand &best, double ts_q, double ts_r, double dt, int kind, int target, int aux, double rate) {
    if (isinf(dt) && dt > 0) return;  // HeapScheduler.push_event ignores infinite times
    Cand c;
    time_add(ts_q, ts_r, dt, c.q, c.r);
    c.kind = kind;
    c.target = target;
    c.aux = aux;
    c.rate = rate;
    if (cand_better(c, best)) best = c;
}

__device__ inline Cand warp_argmin(Cand c) {
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) {
        Cand o;
        o.q = __shfl_xor_sync(kFull, c.q, offset);
        o.r = __shfl_xor_sync(kFull, c.r, offset);
        o.kind = __shfl_xor_sync(kFull, c.kind, offset);
        o.target = __shfl_xor_sync(kFull, c.target, offset);
        o.aux = __shfl_xor_sync(kFull, c.aux, offset);
        o.rate = __shfl_xor_sync(kFull, c.rate, offset);
        if (cand_better(o, c)) c = o;
    }
    return c;
}

__device__ inline int warp_max_int(int v) {
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) v = max(v, __shfl_xor_sync(kFull, v, offset));
    return v;
}

__device__ inline int warp_sum_int(int v) {
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) v += __shfl_xor_sync(kFull, v, offset);
    return v;
}

__device__ inline float warp_min_float(float v) {
#pragma unroll
    for (int offset = 16; offset > 0; offset >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, offset));
    return v;
}

// lifting state of one chain while it runs; lane 0 writes, all lanes read after __syncwarp
struct WarpState {
    double pa[3];
    double ts_q, ts_r, eoc_q, eoc_r;
    double lift_sum;
    long long events, warnings, fallbacks, candidates, refined, liftings, far_lookups;
    int active, direction, eoc_new, occ_active, occ_cell, n_surplus, status, stop;
    // the merged-image thinning derivative of the event against unit real_target, when the warp computed it
    double real_value = 0.0;
    int real_target = -1;
    // cell-veto draws solved ahead by the lanes of a chain's group (coulomb_group_kernel): the first event they
    // cover (-1: none), and the direction and signed charge factor they assumed
    long long spec_base = -1;
    int spec_d = -1;
    double spec_factor = 0.0;
};

struct RunArgs {
    EngineView view;
    double *positions;
    float4 *positions32;
    const double *charges;
    int32_t *occupancy;
    int32_t *surplus;
    int32_t *roles;
    float4 *cell_slots;  // cell-ordered FP32 mirror of the occupancy (x, y, z, identifier bits; bits -1 empty)
    JfgpuChainState *state;
    JfgpuEvent *log;
    long long log_capacity;
    long long first_chain, count, max_events;
    double stop_q, stop_r;
    int has_stop;
    int refine_limit;  // refine lists longer than this re-solve their event in FP64 (1 .. kRefineMax)
    struct FarAhead *ahead;  // [n_chains] the far units' smallest keyed draws of each chain's next event
    int32_t *settle;         // [n_chains] inputs of the chain's settle that have arrived this round (0 between)
};

// int(x / side) along one axis (cuboid_cells.py:190-211), evaluated exactly without a division: the exact float
// bounds of the cells satisfy cell_min[i] <= x <= cell_max[i] if and only if int(x / side) == i, so a multiply by
// 1 / side guesses the index and at most a step or two against the bounds corrects it.
// The compares are taken on the bit patterns, which order the non-negative doubles as integers (no FP64 compare):
// x < 0, -0.0, NaN and x >= L take the division, which gives the same index as before.
__device__ inline long long axis_index(const EngineView &v, const ChainDev &ch, double x) {
    const long long bx = (long long)double_bits(x);
    if (bx < 0 || bx >= (long long)double_bits(ch.L)) return (long long)(x / ch.side);
    const double *lo = v.cell_min + ch.geom_offset;
    const double *hi = v.cell_max + ch.geom_offset;
    long long i = (long long)(x * ch.inv_side);
    if (i > ch.m - 1) i = ch.m - 1;
    if (i < 0) i = 0;
    while (i > 0 && bx < (long long)double_bits(lo[i])) --i;
    while (bx > (long long)double_bits(hi[i])) {
        if (i == ch.m - 1) return ch.m;
        ++i;
    }
    return i;
}

__device__ inline int cell_of(const EngineView &v, const ChainDev &ch, const double *p, int &cell) {
    long long ix = axis_index(v, ch, p[0]), iy = axis_index(v, ch, p[1]), iz = axis_index(v, ch, p[2]);
    long long idx = ix + (long long)ch.m * iy + (long long)ch.m * ch.m * iz;
    if (idx < 0 || idx >= ch.ncells) return JFGPU_STATUS_CELL_RANGE;
    cell = (int)idx;
    return JFGPU_STATUS_OK;
}

__device__ inline void cell_axes(const ChainDev &ch, int cell, int *a) {
    a[0] = cell % ch.m;
    a[1] = (cell / ch.m) % ch.m;
    a[2] = cell / (ch.m * ch.m);
}

__device__ inline bool is_nearby(const ChainDev &ch, int cell, int reference) {
    int a[3], b[3];
    cell_axes(ch, cell, a);
    cell_axes(ch, reference, b);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int diff = a[k] - b[k];
        if (diff < 0) diff += ch.m;
        if (!((ch.near_mask >> diff) & 1ull)) return false;
    }
    return true;
}

__device__ inline int relative_cell(const EngineView &v, const ChainDev &ch, int cell, int reference) {
    int a[3], b[3];
    cell_axes(ch, cell, a);
    cell_axes(ch, reference, b);
    const int16_t *rel = v.rel + ch.table_offset;
    return rel[a[0] * ch.m + b[0]] + ch.m * rel[a[1] * ch.m + b[1]] + ch.m * ch.m * rel[a[2] * ch.m + b[2]];
}

__device__ inline int translate_cell(const EngineView &v, const ChainDev &ch, int cell, int relative) {
    int a[3], b[3];
    cell_axes(ch, cell, a);
    cell_axes(ch, relative, b);
    const int16_t *tra = v.tra + ch.table_offset;
    return tra[a[0] * ch.m + b[0]] + ch.m * tra[a[1] * ch.m + b[1]] + ch.m * ch.m * tra[a[2] * ch.m + b[2]];
}

__device__ inline void separation64(const ChainDev &ch, const double *from, const double *to, double *s) {
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] = py_mod_near((to[k] - from[k]) + ch.half, ch.L) - ch.half;
}

__device__ inline void load_pos(const RunArgs &A, const ChainDev &ch, int j, double *p) {
    const double *q = A.positions + 3 * (ch.pos_off + j);
    p[0] = q[0];
    p[1] = q[1];
    p[2] = q[2];
}

__device__ inline double charge_of(const RunArgs &A, const ChainDev &ch, int j) {
    return A.charges ? A.charges[ch.pos_off + j] : 1.0;
}

// x / speed and x * speed: exact no-ops for the unit speed of the reference's configurations
__device__ inline double div_speed(const ChainDev &ch, double x) { return ch.speed == 1.0 ? x : x / ch.speed; }
__device__ inline double mul_speed(const ChainDev &ch, double x) { return ch.speed == 1.0 ? x : x * ch.speed; }

// keyed draws of one event and kind: the Weyl state key + (counter + 1) * golden with counter = base | target,
// split so that the per-target part is one multiply (same bits as draw())
__device__ inline uint64_t draw_base(uint64_t key, uint64_t event, uint32_t kind) {
    return key + (((event << 24) | ((uint64_t)(kind & 0xFu) << 20)) + 1) * kGolden;
}
__device__ inline uint64_t draw_at(uint64_t base, uint32_t target) {
    return mix64(base + (uint64_t)(target & 0xFFFFFu) * kGolden);
}

// FP64 candidates of one (active, target) pair of the nearby / surplus taggers, one function per potential
__device__ JF_FLOW int exact_pair_hs(const RunArgs &A, const ChainDev &ch, const WarpState &w, int j,
                                         Cand &best) {
    double pj[3], s[3], dt;
    load_pos(A, ch, j, pj);
    separation64(ch, w.pa, pj, s);
    JF_TRY(hs_displacement_axis(ch.diameter_sq, w.direction, ch.speed, s, dt));
    offer(best, w.ts_q, w.ts_r, dt, JFGPU_EV_PAIR, j, -1, 0.0);
    return JFGPU_STATUS_OK;
}

__device__ JF_FLOW int exact_pair_lj(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                         const WarpState &w, int j, long long ev, Cand &best) {
    double pj[3], s[3], disp;
    load_pos(A, ch, j, pj);
    separation64(ch, w.pa, pj, s);
    double du = expovariate(draw(ch.key, (uint64_t)ev, kRngPair, (uint32_t)j), ch.beta);
    JF_TRY(mh_std_displacement(sp.lj, w.direction, s, du, disp));
    offer(best, w.ts_q, w.ts_r, div_speed(ch, disp), JFGPU_EV_PAIR, j, -1, 0.0);
    return JFGPU_STATUS_OK;
}

__device__ JF_FLOW int exact_pair_coulomb(const RunArgs &A, const ChainDev &ch, const WarpState &w, int j,
                                              long long ev, Cand &best) {
    double pj[3], s[3], dt;
    load_pos(A, ch, j, pj);
    separation64(ch, w.pa, pj, s);
    const int d = w.direction;
    if (ch.diameter_sq > 0.0) {
        double sh[3] = {s[0], s[1], s[2]};
        JF_TRY(hs_displacement_axis(ch.diameter_sq, d, ch.speed, sh, dt));
        offer(best, w.ts_q, w.ts_r, dt, JFGPU_EV_HARDCORE, j, -1, 0.0);
    }
    double du = expovariate(draw(ch.key, (uint64_t)ev, kRngPair, (uint32_t)j), ch.beta);
    double p[3];
    permute3(s, d, p);
    double pp = ch.bound_prefactor * charge_of(A, ch, w.active) * charge_of(A, ch, j);
    double disp = ipcb_x_displacement(pp, p[0], p[1], p[2], du, ch.L);
    offer(best, w.ts_q, w.ts_r, div_speed(ch, disp), JFGPU_EV_BOUNDED, j, -1, 0.0);
    return JFGPU_STATUS_OK;
}

// potential and far field of a chain: compile-time constants of a specialised kernel, else read from the chain
template <int POT>
__device__ inline int potential_of(const ChainDev &ch) { return POT >= 0 ? POT : ch.potential; }
template <int FAR>
__device__ inline int far_of(const ChainDev &ch) { return FAR >= 0 ? FAR : ch.far; }

template <int POT>
__device__ inline int exact_pair(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, const WarpState &w,
                                 int j, long long ev, Cand &best) {
    const int pot = potential_of<POT>(ch);
    if (pot == JFGPU_POT_HARD_SPHERE) return exact_pair_hs(A, ch, w, j, best);
    if (pot == JFGPU_POT_LENNARD_JONES) return exact_pair_lj(A, ch, sp, w, j, ev, best);
    return exact_pair_coulomb(A, ch, w, j, ev, best);
}

// FP64 candidate of a far occupant under the cell-bounding potential (cells from the positions, as the handler)
__device__ JF_FLOW int exact_cell_bounding(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                               const WarpState &w, int j, int active_cell, long long ev, Cand &best) {
    double pj[3];
    int target_cell;
    load_pos(A, ch, j, pj);
    JF_TRY(cell_of(A.view, ch, pj, target_cell));
    int rc = relative_cell(A.view, ch, target_cell, active_cell);
    double du = expovariate(draw(ch.key, (uint64_t)ev, kRngPair, (uint32_t)j), ch.beta);
    double rate = sp.bound_upper[rc * 3 + w.direction];
    double disp = rate > 0 ? du / rate : kInf;
    offer(best, w.ts_q, w.ts_r, div_speed(ch, disp), JFGPU_EV_CELL_BOUNDING, j, rc, rate);
    return JFGPU_STATUS_OK;
}

// cell veto, cell boundary and end of chain: the single candidates of lane 0
// the cell-boundary candidate (cell_boundary_event_handler.py:98-156) of the active unit at coordinate x along the
// direction d in cell column a (along d), and the persistent end-of-chain candidate
__device__ inline void boundary_and_end(const EngineView &view, const ChainDev &ch, int d, int a, double x, double ts_q,
                                        double ts_r, double eoc_q, double eoc_r, int eoc_new, Cand &best) {
    const double boundary = view.cell_min[ch.geom_offset + (a + 1 == ch.m ? 0 : a + 1)];
    double sep = boundary - x;
    if (sep < 0.0) sep = sep + ch.L;
    offer(best, ts_q, ts_r, div_speed(ch, sep), JFGPU_EV_BOUNDARY, -1, -1, boundary);
    Cand e;
    e.q = eoc_q;
    e.r = eoc_r;
    e.kind = JFGPU_EV_END_OF_CHAIN;
    e.target = eoc_new;
    e.aux = -1;
    e.rate = 0.0;
    if (cand_better(e, best)) best = e;
}

__device__ JF_FLOW int single_candidates(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                             const WarpState &w, int active_cell, long long ev, Cand &best) {
    const int d = w.direction;
    if (ch.far == JFGPU_FAR_CELL_VETO) {
        double charge_factor = ch.potential == JFGPU_POT_LENNARD_JONES ? 1.0 : (charge_of(A, ch, w.active) * 1.0) / 1.0;
        int which = 0;
        if (!(charge_factor > 0.0)) {
            charge_factor *= -1.0;
            which = 1;
        }
        const WalkerDev &wk = sp.walker[which][d];
        double total_rate = wk.total_rate * charge_factor;
        int k = (int)randbelow(draw(ch.key, (uint64_t)ev, kRngVetoChoice, 0), (uint32_t)wk.size);
        double u = wk.mean_rate * uniform53(draw(ch.key, (uint64_t)ev, kRngVetoUniform, 0));
        int rc = (u <= wk.first_rate[k]) ? wk.first_item[k] : wk.second_item[k];
        double rate = (which == 0 ? sp.bound_upper[rc * 3 + d] : sp.bound_lower[rc * 3 + d]) * charge_factor;
        if (!(rate > 0.0)) return JFGPU_STATUS_ASSERTION;
        int target_cell = translate_cell(A.view, ch, active_cell, rc);
        double dt = expovariate(draw(ch.key, (uint64_t)ev, kRngVetoTime, 0), ch.beta) / mul_speed(ch, total_rate);
        offer(best, w.ts_q, w.ts_r, dt, JFGPU_EV_CELL_VETO, -1, target_cell, rate);
    }
    int ax[3];
    cell_axes(ch, active_cell, ax);
    boundary_and_end(A.view, ch, d, ax[d], w.pa[d], w.ts_q, w.ts_r, w.eoc_q, w.eoc_r, w.eoc_new, best);
    return JFGPU_STATUS_OK;
}

// ---------------------------------------------------------------------------------------------------------------
// occupancy (lane 0)
// ---------------------------------------------------------------------------------------------------------------
// role word of a unit: the axes of its occupancy cell (x | y << 8 | z << 16); for a surplus unit bit 24 and its
// index in the chain's surplus list instead of the axes; bit 25 for the occupancy's active unit
constexpr int32_t kRoleSurplus = 1 << 24;
constexpr int32_t kRoleActive = 1 << 25;

__device__ inline int32_t role_of_cell(const ChainDev &ch, int cell) {
    int a[3];
    cell_axes(ch, cell, a);
    return a[0] | (a[1] << 8) | (a[2] << 16);
}

// the cell slot of occupancy entry `slot` holds the occupant's FP32 mirror position and identifier (or -1)
__device__ inline void set_cell_slot(const RunArgs &A, long long slot, int id, const float4 &p) {
    A.cell_slots[slot] = make_float4(p.x, p.y, p.z, __int_as_float(id));
}

__device__ inline void occ_insert(const RunArgs &A, const ChainDev &ch, WarpState &w, int cell, int id) {
    int32_t *slots = A.occupancy + ch.occ_off + (long long)cell * ch.max_occ;
    for (int k = 0; k < ch.max_occ; ++k)
        if (slots[k] < 0) {
            slots[k] = id;
            A.roles[ch.pos_off + id] = role_of_cell(ch, cell);
            set_cell_slot(A, ch.occ_off + (long long)cell * ch.max_occ + k, id, A.positions32[ch.pos_off + id]);
            return;
        }
    A.surplus[ch.pos_off + w.n_surplus] = id;
    A.roles[ch.pos_off + id] = kRoleSurplus | w.n_surplus;
    w.n_surplus += 1;
}

__device__ JF_FLOW int occ_update(const RunArgs &A, const ChainDev &ch, WarpState &w) {
    if (w.active != w.occ_active) {
        const int32_t role = A.roles[ch.pos_off + w.active];
        if (w.occ_active >= 0) occ_insert(A, ch, w, w.occ_cell, w.occ_active);
        if (role & (kRoleSurplus | kRoleActive)) {
            JF_TRY(cell_of(A.view, ch, w.pa, w.occ_cell));
        } else {
            // an occupant has not moved since it entered its cell (only the active unit moves): the cell of its
            // position is the one its role word names
            w.occ_cell = (role & 0xFF) + ch.m * (((role >> 8) & 0xFF) + ch.m * ((role >> 16) & 0xFF));
        }
        w.occ_active = w.active;
        A.roles[ch.pos_off + w.active] = kRoleActive;
        int32_t *slots = A.occupancy + ch.occ_off + (long long)w.occ_cell * ch.max_occ;
        for (int k = 0; k < ch.max_occ; ++k)
            if (slots[k] == w.active) {
                slots[k] = -1;
                set_cell_slot(A, ch.occ_off + (long long)w.occ_cell * ch.max_occ + k, -1, make_float4(0.f, 0.f, 0.f, 0.f));
                return JFGPU_STATUS_OK;
            }
        // a surplus unit: its role word (read before it was overwritten above) holds its index in the list;
        // the last entry moves into its place (SingleActiveCellOccupancy._surplus keeps no order)
        int32_t *sur = A.surplus + ch.pos_off;
        if (!(role & kRoleSurplus)) return JFGPU_STATUS_ASSERTION;
        const int k = role & 0xFFFFFF;
        if (k >= w.n_surplus || sur[k] != w.active) return JFGPU_STATUS_ASSERTION;
        const int last = sur[w.n_surplus - 1];
        sur[k] = last;
        if (last != w.active) A.roles[ch.pos_off + last] = kRoleSurplus | k;
        w.n_surplus -= 1;
        return JFGPU_STATUS_OK;
    }
    return cell_of(A.view, ch, w.pa, w.occ_cell);
}

// ---------------------------------------------------------------------------------------------------------------
// out-state (lane 0)
// ---------------------------------------------------------------------------------------------------------------
__device__ inline int real_rate(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, const WarpState &w, int t,
                                double &out) {
    double pt[3], s[3];
    load_pos(A, ch, t, pt);
    separation64(ch, w.pa, pt, s);
    if (ch.potential == JFGPU_POT_LENNARD_JONES) {
        double value;
        JF_TRY(mh_std_derivative(sp.lj, w.direction, s, value));
        out = mul_speed(ch, value);
        return JFGPU_STATUS_OK;
    }
    if (w.real_target == t) {  // shared by the warp before the commit (warp_real_rate)
        out = w.real_value;
        return JFGPU_STATUS_OK;
    }
    out = mul_speed(ch, mic_std_derivative(sp.mic, ch.coulomb_prefactor, w.direction, s, charge_of(A, ch, w.active),
                                           charge_of(A, ch, t)));
    return JFGPU_STATUS_OK;
}

// The thinning derivative of a merged-image Coulomb event (bounded pair or cell veto with an occupant) computed by
// the whole warp before lane 0 commits it: the target and the time-sliced active position as the commit will have
// them, the sum shared by the lanes (mic_x_warp: the serial sum's terms in another order of additions, within
// 1e-12).  Every lane calls it; lane 0 stores the value for real_rate.
__device__ inline void warp_real_rate(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w,
                                      const Cand &best, int lane) {
    int t = -1;
    double pa[3] = {0.0, 0.0, 0.0};
    if (lane == 0) {
        w.real_target = -1;
        if (best.kind == JFGPU_EV_BOUNDED)
            t = best.target;
        else if (best.kind == JFGPU_EV_CELL_VETO)
            t = A.occupancy[ch.occ_off + (long long)best.aux * ch.max_occ];
        if (t >= 0) {
            const double dt = time_sub(best.q, best.r, w.ts_q, w.ts_r);  // as time_slice
            for (int k = 0; k < 3; ++k) pa[k] = w.pa[k];
            pa[w.direction] = py_mod_near(w.pa[w.direction] + ch.speed * dt, ch.L);
        }
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t < 0) return;
    for (int k = 0; k < 3; ++k) pa[k] = __shfl_sync(0xffffffffu, pa[k], 0);
    double pt[3], s[3], p[3];
    load_pos(A, ch, t, pt);
    separation64(ch, pa, pt, s);
    permute3(s, w.direction, p);
    CompositeModel model;
    model.mic = sp.mic;
    model.images = sp.mic_terms;
    model.n_images = sp.mic_images;
    model.rows = sp.mic_terms + sp.mic_images;
    model.n_rows = sp.mic_rows;
    const double value = mic_x_warp(model, p[0], p[1], p[2], lane);
    if (lane == 0) {
        w.real_value = mul_speed(ch, ch.coulomb_prefactor * charge_of(A, ch, w.active) * charge_of(A, ch, t) * value);
        w.real_target = t;
    }
}

// Thinning: accept iff uniform(0, bound) < real rate (event_handler_with_bounding_potential.py:95-101).  For
// Lennard-Jones the decision (and the bound-violation count) is first taken in FP32 from the FP32 mirror; only a
// decision within the FP32 error margin is re-taken in FP64, so the outcome always equals the FP64 one.
__device__ JF_FLOW int thinning(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w, int t,
                                    double bounding_rate, long long ev, int &accepted) {
    const double u = uniform53(draw(ch.key, (uint64_t)ev, kRngThin, 0));
    if (ch.potential == JFGPU_POT_LENNARD_JONES) {
        const float4 pt = A.positions32[ch.pos_off + t];
        float sv[3] = {pt.x - (float)w.pa[0], pt.y - (float)w.pa[1], pt.z - (float)w.pa[2]};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (sv[k] >= ch.half32) sv[k] -= ch.L32;
            if (sv[k] < -ch.half32) sv[k] += ch.L32;
        }
        const float r2 = sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2];
        const float ir2 = 1.0f / r2;
        const float ir8 = ir2 * ir2 * ir2 * ir2;
        const float ir14 = ir8 * ir2 * ir2 * ir2;
        const float c6 = (float)(6.0 * sp.lj.six.prefactor) * ir8;
        const float c12 = (float)(12.0 * sp.lj.twelve.prefactor) * ir14;
        const float speed = (float)ch.speed;
        const float sd = sv[w.direction];
        const float real32 = (c6 + c12) * sd * speed;
        const float bound32 = (float)bounding_rate;
        const float ub32 = bound32 * (float)u;
        const float scale = (fabsf(c6) + fabsf(c12)) * speed;
        const float margin = scale * (fabsf(sd) * (1.0f / 1024.0f) + 64.0f * ch.ulp_margin32) + ub32 * (1.0f / 65536.0f) +
                             bound32 * (1.0f / 65536.0f);
        const bool ambiguous = !(fabsf(real32 - ub32) > margin) || !(fabsf(bound32 - real32) > margin) ||
                               !isfinite(real32);
        if (!ambiguous) {
            accepted = real32 > ub32 ? 1 : 0;
            if (real32 > 0.0f && bound32 < real32) w.warnings += 1;
            return JFGPU_STATUS_OK;
        }
    }
    double real;
    JF_TRY(real_rate(A, ch, sp, w, t, real));
    accepted = 0;
    if (real > 0) {
        if (bounding_rate < real) w.warnings += 1;
        if (bounding_rate * u < real) accepted = 1;
    }
    return JFGPU_STATUS_OK;
}

__device__ inline void store_active(const RunArgs &A, const ChainDev &ch, const WarpState &w, int id) {
    double *q = A.positions + 3 * (ch.pos_off + id);
    q[0] = w.pa[0];
    q[1] = w.pa[1];
    q[2] = w.pa[2];
    float *m = reinterpret_cast<float *>(A.positions32 + ch.pos_off + id);  // x, y, z; the charge stays
    m[0] = (float)w.pa[0];
    m[1] = (float)w.pa[1];
    m[2] = (float)w.pa[2];
}

// BasicEventHandler._time_slice_unit (abstracts.py:82-95): position[d] = (position[d] + v[d] * dt) % L.  For the
// components of zero velocity this is p + 0.0 * dt then p % L, which returns p exactly for p in [0, L).
__device__ inline void time_slice(const ChainDev &ch, WarpState &w, double q, double r) {
    double dt = time_sub(q, r, w.ts_q, w.ts_r);
    const int d = w.direction;
    w.pa[d] = py_mod_near(w.pa[d] + ch.speed * dt, ch.L);
    w.ts_q = q;
    w.ts_r = r;
}

// commit the winner; returns a status
__device__ JF_FLOW int commit(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w, const Cand &best,
                             int active_cell, long long chain_index, long long log_index) {
    // the data of the commit and of the occupancy update after it, requested together so that their latencies
    // overlap the time slice: the cell's slots, and the new active unit's position and role word
    asm volatile("prefetch.global.L1 [%0];" ::"l"(A.occupancy + ch.occ_off + (long long)active_cell * ch.max_occ));
    if (best.target >= 0 && best.target < ch.n) {
        asm volatile("prefetch.global.L1 [%0];" ::"l"(A.positions + 3 * (ch.pos_off + best.target)));
        asm volatile("prefetch.global.L1 [%0];" ::"l"(A.roles + ch.pos_off + best.target));
    }
    const long long ev = w.events;
    int moved = w.active;
    JfgpuEvent rec;
    rec.kind = best.kind;
    rec.moved = moved;
    rec.target = -1;
    rec.accepted = 0;
    rec.time_q = best.q;
    rec.time_r = best.r;
    time_slice(ch, w, best.q, best.r);
    switch (best.kind) {
    case JFGPU_EV_PAIR:
    case JFGPU_EV_HARDCORE:
        rec.target = best.target;
        rec.accepted = 1;
        w.active = best.target;
        break;
    case JFGPU_EV_BOUNDED: {
        double pt[3], s[3], p[3];
        load_pos(A, ch, best.target, pt);
        separation64(ch, w.pa, pt, s);
        permute3(s, w.direction, p);
        double pp = ch.bound_prefactor * charge_of(A, ch, w.active) * charge_of(A, ch, best.target);
        double bound = mul_speed(ch, ipcb_x_derivative(pp, p[0], p[1], p[2]));
        int accepted;
        JF_TRY(thinning(A, ch, sp, w, best.target, bound, ev, accepted));
        rec.target = best.target;
        rec.accepted = accepted;
        if (accepted) w.active = best.target;
        break;
    }
    case JFGPU_EV_CELL_BOUNDING: {
        int now_cell;
        JF_TRY(cell_of(A.view, ch, w.pa, now_cell));
        if (now_cell != active_cell) return JFGPU_STATUS_ASSERTION;
        int accepted;
        JF_TRY(thinning(A, ch, sp, w, best.target, mul_speed(ch, best.rate), ev, accepted));
        rec.target = best.target;
        rec.accepted = accepted;
        if (accepted) w.active = best.target;
        break;
    }
    case JFGPU_EV_CELL_VETO: {
        int t = A.occupancy[ch.occ_off + (long long)best.aux * ch.max_occ];
        if (t >= 0) {
            int accepted;
            JF_TRY(thinning(A, ch, sp, w, t, best.rate, ev, accepted));
            rec.target = t;
            rec.accepted = accepted;
            if (accepted) w.active = t;
        }
        break;
    }
    case JFGPU_EV_BOUNDARY:
        w.pa[w.direction] = best.rate;
        break;
    case JFGPU_EV_END_OF_CHAIN: {
        w.direction = (w.direction + 1) % 3;
        w.active = best.target;
        rec.target = best.target;
        rec.accepted = 1;
        time_add(w.ts_q, w.ts_r, time_sub(w.ts_q, w.ts_r, w.ts_q, w.ts_r) + ch.chain_time, w.eoc_q, w.eoc_r);
        w.eoc_new = (int)randbelow(draw(ch.key, (uint64_t)(ev + 1), kRngNewActive, 0), (uint32_t)ch.n);
        break;
    }
    default:
        return JFGPU_STATUS_ASSERTION;
    }
    rec.new_active = w.active;
    rec.new_direction = w.direction;
    rec.x = w.pa[0];
    rec.y = w.pa[1];
    rec.z = w.pa[2];
    store_active(A, ch, w, moved);
    if (w.active != moved) {
        double pn[3];
        load_pos(A, ch, w.active, pn);
        if (best.kind != JFGPU_EV_END_OF_CHAIN) {
            // excess displacement of the lifting: separation target - active along the (unchanged) direction
            const int d = w.direction;
            w.lift_sum += py_mod_near((pn[d] - w.pa[d]) + ch.half, ch.L) - ch.half;
            w.liftings += 1;
        }
        w.pa[0] = pn[0];
        w.pa[1] = pn[1];
        w.pa[2] = pn[2];
    }
    if (A.log && log_index < A.log_capacity) A.log[(chain_index - A.first_chain) * A.log_capacity + log_index] = rec;
    w.events = ev + 1;
    return JFGPU_STATUS_OK;
}

// out-of-line entry points of the event flow for the warp-per-chain FP64 kernel (chains_kernel) and the rare serial
// re-solve of a whole event, which call it from several places
template <int POT>
__device__ __noinline__ int exact_pair_ool(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                           const WarpState &w, int j, long long ev, Cand &best) {
    return exact_pair<POT>(A, ch, sp, w, j, ev, best);
}
__device__ __noinline__ int exact_cell_bounding_ool(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                                    const WarpState &w, int j, int active_cell, long long ev,
                                                    Cand &best) {
    return exact_cell_bounding(A, ch, sp, w, j, active_cell, ev, best);
}
__device__ __noinline__ int single_candidates_ool(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                                  const WarpState &w, int active_cell, long long ev, Cand &best) {
    return single_candidates(A, ch, sp, w, active_cell, ev, best);
}
__device__ __noinline__ int commit_ool(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w,
                                       const Cand &best, int active_cell, long long chain_index, long long log_index) {
    return commit(A, ch, sp, w, best, active_cell, chain_index, log_index);
}
__device__ __noinline__ int occ_update_ool(const RunArgs &A, const ChainDev &ch, WarpState &w) {
    return occ_update(A, ch, w);
}

// ---------------------------------------------------------------------------------------------------------------
// candidate enumeration
// ---------------------------------------------------------------------------------------------------------------

// base-K digits (x, y, z) of lane + step k (step 32 by default), advanced without divisions (K >= 1, step <= 32; one
// carry per digit)
struct Digits {
    int x, y, z, sx, sy, sz, K;
    __device__ inline void start(int lane, int base, int step = 32) {
        K = base;
        x = lane % K;
        y = (lane / K) % K;
        z = lane / (K * K);
        sx = step % K;
        sy = (step / K) % K;
        sz = step / (K * K);
    }
    __device__ inline void advance() {
        x += sx;
        y += sy;
        z += sz;
        if (x >= K) {
            x -= K;
            ++y;
        }
        if (y >= K) {
            y -= K;
            ++z;
        }
    }
};

// occupants of the nearby cells of the occupancy's active cell (ExcludedCellsTagger), lane `lane` of `step` lanes
template <typename F>
__device__ inline void for_each_near(const RunArgs &A, const ChainDev &ch, int occ_cell, int lane, F &&f,
                                     int step = 32) {
    int a[3];
    cell_axes(ch, occ_cell, a);
    const int K = ch.n_res;
    const int32_t *occ = A.occupancy + ch.occ_off;
    Digits g;
    g.start(lane, K, step);
    for (; g.z < K; g.advance()) {
        int cx = a[0] + ch.res[g.x], cy = a[1] + ch.res[g.y], cz = a[2] + ch.res[g.z];
        if (cx >= ch.m) cx -= ch.m;
        if (cy >= ch.m) cy -= ch.m;
        if (cz >= ch.m) cz -= ch.m;
        const int cell = cx + ch.m * (cy + ch.m * cz);
        for (int k = 0; k < ch.max_occ; ++k) {
            int j = occ[(long long)cell * ch.max_occ + k];
            if (j >= 0) f(j);
        }
    }
}

// occupants of the cells that are not nearby (CellBoundingPotentialTagger), with their relative cell
template <typename F>
__device__ inline void for_each_far(const RunArgs &A, const ChainDev &ch, int occ_cell, int lane, F &&f) {
    int a[3];
    cell_axes(ch, occ_cell, a);
    const int m = ch.m;
    const int32_t *occ = A.occupancy + ch.occ_off;
    const int16_t *rel = A.view.rel + ch.table_offset;
    Digits g;
    g.start(lane, m);
    for (; g.z < m; g.advance()) {
        const int cell = g.x + m * (g.y + m * g.z);
        const int j = occ[cell];
        if (j < 0) continue;
        int dx = g.x - a[0], dy = g.y - a[1], dz = g.z - a[2];
        if (dx < 0) dx += m;
        if (dy < 0) dy += m;
        if (dz < 0) dz += m;
        if (((ch.near_mask >> dx) & 1ull) && ((ch.near_mask >> dy) & 1ull) && ((ch.near_mask >> dz) & 1ull)) continue;
        int rc;
        if (ch.rel_is_mod) {
            rc = dx + m * (dy + m * dz);
        } else {
            rc = rel[g.x * m + a[0]] + m * (rel[g.y * m + a[1]] + m * rel[g.z * m + a[2]]);
        }
        f(j, cell, rc);
    }
}

// Every non-active unit with its role word (from `roles`, the chain's role array in global or shared memory; the
// cell-bounding far field makes every unit a candidate): surplus units and
// occupants of nearby cells go to `near(j)`, occupants of the other cells to `far(j, rc)` with their relative cell.
// The same partition as the taggers (ExcludedCellsTagger, SurplusCellsTagger, CellBoundingPotentialTagger), found by
// one coalesced pass over the units instead of two passes over the cells.
template <typename FN, typename FF>
__device__ inline void for_each_unit(const int32_t *roles, const RunArgs &A, const ChainDev &ch, int occ_cell, int lane,
                                     FN &&near, FF &&far) {
    int a[3];
    cell_axes(ch, occ_cell, a);
    const int m = ch.m;
    const int16_t *rel = A.view.rel + ch.table_offset;
    for (int j = lane; j < ch.n; j += 32) {
        const int32_t role = roles[j];
        if (role & kRoleActive) continue;
        if (role & kRoleSurplus) {
            near(j);
            continue;
        }
        const int cx = role & 0xFF, cy = (role >> 8) & 0xFF, cz = (role >> 16) & 0xFF;
        int dx = cx - a[0], dy = cy - a[1], dz = cz - a[2];
        if (dx < 0) dx += m;
        if (dy < 0) dy += m;
        if (dz < 0) dz += m;
        if (((ch.near_mask >> dx) & 1ull) && ((ch.near_mask >> dy) & 1ull) && ((ch.near_mask >> dz) & 1ull)) {
            near(j);
            continue;
        }
        const int rc = ch.rel_is_mod ? dx + m * (dy + m * dz)
                                     : rel[cx * m + a[0]] + m * (rel[cy * m + a[1]] + m * rel[cz * m + a[2]]);
        far(j, rc);
    }
}

// the whole event in FP64 (all lanes); returns the winner in best
template <int POT, int FAR>
__device__ inline int exact_candidates(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, const WarpState &w,
                                       int active_cell, int lane, Cand &best, int &counted) {
    const long long ev = w.events;
    int status = JFGPU_STATUS_OK;
    int count = 0;
    best = cand_none();
    for_each_near(A, ch, w.occ_cell, lane, [&](int j) {
        int st = exact_pair_ool<POT>(A, ch, sp, w, j, ev, best);
        if (st) status = st;
        ++count;
    });
    for (int i = lane; i < w.n_surplus; i += 32) {
        int st = exact_pair_ool<POT>(A, ch, sp, w, A.surplus[ch.pos_off + i], ev, best);
        if (st) status = st;
        ++count;
    }
    counted = warp_sum_int(count);
    if (far_of<FAR>(ch) == JFGPU_FAR_CELL_BOUNDING) {
        for_each_far(A, ch, w.occ_cell, lane, [&](int j, int cell, int rc) {
            int st = exact_cell_bounding_ool(A, ch, sp, w, j, active_cell, ev, best);
            if (st) status = st;
        });
    }
    if (lane == 0) {
        int st = single_candidates_ool(A, ch, sp, w, active_cell, ev, best);
        if (st) status = st;
    }
    best = warp_argmin(best);
    return warp_max_int(status);
}

// top-K insertion of (key, code) pairs kept sorted ascending
__device__ inline void topk_insert(float (&key)[kTopK], int (&code)[kTopK], float k, int c) {
    if (!(k < key[kTopK - 1])) return;
    key[kTopK - 1] = k;
    code[kTopK - 1] = c;
#pragma unroll
    for (int i = kTopK - 1; i > 0; --i) {
        if (key[i] < key[i - 1]) {
            float tk = key[i];
            key[i] = key[i - 1];
            key[i - 1] = tk;
            int tc = code[i];
            code[i] = code[i - 1];
            code[i - 1] = tc;
        }
    }
}

__device__ inline float lane_min_unflagged(const float (&key)[kTopK]) {
    float v = kInf32;
#pragma unroll
    for (int i = 0; i < kTopK; ++i)
        if (key[i] >= 0.0f) v = fminf(v, key[i]);
    return v;
}

// ---------------------------------------------------------------------------------------------------------------
// Mixed precision as a two-phase event.
//   screen_kernel (one warp per chain, FP32 only): every candidate is screened in FP32; the candidates within
//                 (1 + 2^-10) t_min + margin, and every flagged one, go to the chain's refine list.
//   settle_kernel (FP64): the listed candidates (one thread each) and the single candidates (cell veto, cell
//                 boundary, end of chain; one thread per chain) are solved with the reference's arithmetic; the
//                 thread that completes a chain's inputs commits the earliest and updates the occupancy for the
//                 next event.
// The FP64 work of 32 chains thus shares each warp instruction, instead of occupying lane 0 of 32 warps, and each
// kernel carries a small instruction footprint.  The winner and its time are the FP64 ones: the mixed path equals
// the FP64 path event for event.
// ---------------------------------------------------------------------------------------------------------------
constexpr int kRefineMax = JFGPU_REFINE_LIST_MAX;
constexpr int32_t kListOverflow = 1;
constexpr int32_t kListSkip = 2;

// list entry: target in bits 0-19, screening path in bits 20-23, bit 30 for a far (cell-bounding) candidate
constexpr int32_t kCodeFar = 1 << 30;
__device__ inline int32_t make_code(int target, int path, bool far) {
    return target | (path << 20) | (far ? kCodeFar : 0);
}
__device__ inline int code_target(int32_t code) { return code & 0xFFFFF; }
__device__ inline int code_path(int32_t code) { return (code >> 20) & 0xF; }
__device__ inline bool code_far(int32_t code) { return (code & kCodeFar) != 0; }

struct RefineList {
    int32_t count, flags, screened, far_lookups;
    int32_t code[kRefineMax];
};

// FP64 re-solves of the first kRefineSlots entries of every refine list, one thread per entry; the thread that
// settles the chain takes the earliest of them (and solves any further entry itself)
#ifndef JF_REFINE_SLOTS
#define JF_REFINE_SLOTS 4
#endif
constexpr int kRefineSlots = JF_REFINE_SLOTS;
constexpr int kQueueHalf = 16;  // a group's 32 queue counters: kPaths of the even rounds, then of the odd ones

// Refine queue of a chain group: per screening path, the entries (local chain * kRefineSlots + slot) to re-solve.
// counts[kPaths] sit in the group's header; entries[path][...] use the slice [lo, hi) * kRefineSlots of the group's
// chains, so that groups on different streams never share a word.
struct RefineQueue {
    int32_t *counts;   // [2][kQueueHalf]: round r fills half r & 1, which the settle kernel of round r - 1 zeroed
    int32_t *entries;  // [kPaths][stride], offset to the group's slice
    long long stride;  // n_chains * kRefineSlots
};

// keyed draw of a pair candidate: only its top 32 bits enter the FP32 screening (uniform within 2^-32)
__device__ inline uint32_t draw_hi32(uint64_t base, uint32_t target) { return (uint32_t)(draw_at(base, target) >> 32); }

// Nearby cells along one axis: the K cells starting at first = a - layers (wrapped), or the whole axis when the layers
// cover it (K = m); the same set as the distinct residues of the layer offsets (cuboid_periodic_cells.py:74-100)
__device__ inline int near_first(int a, int K, int m) {
    if (K == m) return 0;
    const int first = a - (K >> 1);
    return first < 0 ? first + m : first;
}

#ifndef JF_NEAR_BATCH
#define JF_NEAR_BATCH 4
#endif
constexpr int kNearBatch = JF_NEAR_BATCH;  // cell slots each lane loads before it screens them (loads in flight)
constexpr int kKeptMax = 96;   // kept nearby and surplus candidates a warp solves in FP32 (more: FP64 path)

// The far units whose keyed pair draws of an event are small, listed before the event: every unit j of the chain
// with u24 = (draw >> 40) < bound, in increasing j, with the top 32 bits of its draw.  The list depends only on the
// chain's key, the event number and the number of units, so a record whose key and event match the screened event
// is that event's list whenever it was made.  The screening kernel of an event writes `next` (the event number
// after it, -1 for a skipped chain); far_ahead_warp lists that event while the round's FP64 kernels run.
constexpr int kAhead = 32;        // listed units at most (one a lane)
constexpr int kAheadExpect = 16;  // expected listed units: bound = ceil(16 * 2^24 / n)
struct FarAhead {
    long long event;  // the listed event (the record is void unless key matches too)
    long long next;   // the event the next far_ahead_warp lists (-1: none)
    uint64_t key;
    uint32_t bound;   // every unlisted unit has u24 >= bound (0: the list overflowed)
    int32_t count;
    int32_t unit[kAhead];
    uint32_t hi[kAhead];
};
__device__ inline uint32_t ahead_bound(int n) {
    const uint64_t b = ((uint64_t)kAheadExpect << 24) / (uint64_t)(n > 0 ? n : 1) + 1;
    return b < (1ull << 24) ? (uint32_t)b : (1u << 24);
}

#ifndef JF_SCREEN_REGS
#define JF_SCREEN_REGS 72
#endif
template <int POT, int FAR>
__global__ void __maxnreg__(JF_SCREEN_REGS) screen_kernel(RunArgs A, RefineList *lists, RefineQueue queue,
                                                         long long round, int first_round) {
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long local = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
    if (local >= A.count) return;
    const long long c = A.first_chain + local;
    const ChainDev &ch = A.view.chains[c];
    const SpeciesDev &sp = A.view.species[ch.species];
    RefineList &list = lists[local];
    const JfgpuChainState &g = A.state[c];
    if (g.status != JFGPU_STATUS_OK || (!first_round && g.stopped)) {
        if (lane == 0) {
            list.count = 0;
            list.flags = kListSkip;
            list.screened = 0;
            list.far_lookups = 0;
            A.ahead[c].next = -1;
        }
        return;
    }
    if (potential_of<POT>(ch) == JFGPU_POT_COULOMB) {
        // merged-image Coulomb chains (a few dozen charges) are solved entirely in FP64 by their resolve thread
        if (lane == 0) {
            list.count = 0;
            list.flags = kListOverflow;
            list.screened = 0;
            list.far_lookups = 0;
        }
        return;
    }
    const int active = g.active, d = g.direction, occ_cell = g.occ_cell, n_surplus = g.n_surplus;
    const int m = ch.m, K = ch.n_res, max_occ = ch.max_occ, n = ch.n;
    const long long pos_off = ch.pos_off, occ_off = ch.occ_off;
    const uint64_t ev = (uint64_t)g.events;
    const float speed32 = ch.speed32;
    const float inv_beta32 = ch.inv_beta32;
    const float margin = ch.ulp_margin32;
    const float L32 = ch.L32, half32 = ch.half32;
    const float rel = 1.0f + 1.0f / 1024.0f;
    const float abs_margin = ch.screen_abs32 / speed32;
    const float4 pa32 = A.positions32[pos_off + active];
    // the chain's far-ahead record (three 128-byte lines), read by the far pass after the nearby scan
    if (far_of<FAR>(ch) == JFGPU_FAR_CELL_BOUNDING && lane < 3)
        asm volatile("prefetch.global.L1 [%0];" ::"l"(reinterpret_cast<const char *>(A.ahead + c) + 128 * lane));
    int ax[3];
    cell_axes(ch, occ_cell, ax);
    // single candidates in FP32 bound the threshold: the cell boundary and the end of chain
    float t_single;
    {
        const int next = ax[d] + 1 == m ? 0 : ax[d] + 1;
        const float boundary = (float)A.view.cell_min[ch.geom_offset + next];
        const float x = d == 0 ? pa32.x : (d == 1 ? pa32.y : pa32.z);
        float sep = boundary - x;
        if (sep < 0.0f) sep += L32;
        t_single = sep / speed32;
        t_single = fminf(t_single, (float)time_sub(g.eoc_q, g.eoc_r, g.time_q, g.time_r));
    }
    LJ32 lj32;
    lj32.a12 = sp.lj32[0];
    lj32.a6 = sp.lj32[1];
    lj32.four_over_k = sp.lj32[2];
    lj32.sigma_sq = sp.lj32[3];
    lj32.r0_sq = sp.lj32[4];
    float key[kTopK];
    int code[kTopK];
#pragma unroll
    for (int i = 0; i < kTopK; ++i) {
        key[i] = kInf32;
        code[i] = -1;
    }
    const uint64_t pair_base = draw_base(ch.key, ev, kRngPair);
    int count = 0;
    // the FP32 solve of a kept candidate (x, y, z, identifier bits)
    auto screen_pair = [&](const float4 &pj) {
        const int j = __float_as_int(pj.w);
        float sv[3];
        bool flag = false;
        separation32(pa32, pj, L32, half32, margin, sv, flag);
        float t;
        int path = kPathHardSphere;
        if (potential_of<POT>(ch) == JFGPU_POT_HARD_SPHERE) {
            t = hs_screen(ch.diameter_sq32, d, speed32, sv, margin, flag);
        } else {
            const float du = expovariate32((uint64_t)draw_hi32(pair_base, (uint32_t)j) << 32, inv_beta32, flag);
            t = lj_screen(lj32, d, speed32, sv, du, margin, flag, path);
        }
        // a flagged candidate keeps the branch its FP32 solve took (the flag concerns the time, rarely the branch):
        // its FP64 re-solve joins the warps of that branch
        if (flag) t = -1.0f;
        if (!isinf(t)) topk_insert(key, code, t, make_code(j, path, false));
    };
    // Pre-test of every nearby occupant and surplus unit: a candidate whose event cannot come before the single
    // candidates (cell boundary, end of chain) is dropped before its logarithm and inversion.  Along the active's
    // move x in [0, D] (D the single candidates' time, padded) the distance to the target is smallest at
    // x* = clamp(s_d, 0, D).  Hard spheres: no contact if that distance exceeds the diameter.  Lennard-Jones: if the
    // whole path stays outside the minimum shell, U rises by at most |U(r_min)| (it falls towards r_min and rises
    // after), and an event needs du = -log(1 - u) / beta <= |U(r_min)|, impossible for u > beta |U(r_min)|.  Both
    // tests carry relative margins far above FP32 rounding.  The kept candidates are compacted per warp so that
    // every lane solves one in each pass.
    const float horizon = (t_single * rel + abs_margin) * speed32;
    const float shell32 = potential_of<POT>(ch) == JFGPU_POT_HARD_SPHERE ? ch.diameter_sq32 : lj32.r0_sq;
    const float beta32 = 1.0f / inv_beta32;
    auto keep = [&](const float4 &pj) -> bool {
        float sv[3];
        bool flag = false;
        separation32(pa32, pj, L32, half32, margin, sv, flag);
        if (flag) return true;
        const float sd = sv[d];
        const float pa = d == 0 ? sv[1] : sv[0];
        const float pb = d == 2 ? sv[1] : sv[2];
        const float x = fminf(fmaxf(sd, 0.0f), horizon);
        const float gap = sd - x;
        const float r_min_sq = __fmaf_rn(gap, gap, __fmaf_rn(pa, pa, pb * pb)) * (1.0f - 1.0f / 4096.0f);
        if (!(r_min_sq > shell32 * (1.0f + 1.0f / 4096.0f))) return true;
        if (potential_of<POT>(ch) == JFGPU_POT_HARD_SPHERE) return false;
        // the approximate reciprocal (1 ulp) and the fused products stay far inside the bound's 2^-10 margin
        float ir2;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ir2) : "f"(r_min_sq));
        const float ir6 = ir2 * ir2 * ir2;
        const float rise = -(__fmaf_rn(lj32.a12, ir6, lj32.a6) * ir6);  // |U(r_min)|, U < 0 outside the shell
        const uint32_t hi = draw_hi32(pair_base, (uint32_t)__float_as_int(pj.w));
        const float u_low = (float)(hi >> 8) * (1.0f / 16777216.0f);
        return !(u_low > beta32 * rise * (1.0f + 1.0f / 1024.0f));
    };
    bool kept_over = false;  // warp-uniform
    {
        // Nearby occupants from the cell-ordered mirror: one 16-byte load gives an occupant's FP32 position and
        // identifier, the cells of a row along x are contiguous, and each lane keeps kNearBatch loads in flight.
        // Kept candidates wait in a per-warp buffer (dynamic shared memory, kKeptMax a warp) and are solved in FP32
        // after the scan, so that the scan's loop carries none of the solve's registers; more than kKeptMax of them
        // send the event to the FP64 path (the refine list's overflow).
        extern __shared__ float4 kept_smem[];
        float4 *buf = kept_smem + warp * kKeptMax;
        int buffered = 0;  // warp-uniform
        auto offer_kept = [&](bool kept, const float4 &pj) {
            const unsigned mask = __ballot_sync(kFull, kept);
            const int at = buffered + __popc(mask & ((1u << lane) - 1u));
            if (kept && at < kKeptMax) buf[at] = pj;
            buffered += __popc(mask);
        };
        const int first_x = near_first(ax[0], K, m), first_y = near_first(ax[1], K, m),
                  first_z = near_first(ax[2], K, m);
        const float4 *slots = A.cell_slots + occ_off;
        const int cell_iters = (K * K * K + 31) / 32;
        for (int slot = 0; slot < max_occ; ++slot) {
            Digits dg;
            dg.start(lane, K);
            for (int it = 0; it < cell_iters; it += kNearBatch) {
                float4 p[kNearBatch];
#pragma unroll
                for (int b = 0; b < kNearBatch; ++b) {
                    p[b] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
                    if (it + b < cell_iters && dg.z < K) {
                        int cx = first_x + dg.x, cy = first_y + dg.y, cz = first_z + dg.z;
                        if (cx >= m) cx -= m;
                        if (cy >= m) cy -= m;
                        if (cz >= m) cz -= m;
                        p[b] = slots[(long long)(cx + m * (cy + m * cz)) * max_occ + slot];
                    }
                    dg.advance();
                }
#pragma unroll
                for (int b = 0; b < kNearBatch; ++b) {
                    if (it + b >= cell_iters) break;  // warp-uniform
                    bool kept = false;
                    if (__float_as_int(p[b].w) >= 0) {
                        ++count;
                        kept = keep(p[b]);
                    }
                    offer_kept(kept, p[b]);
                }
            }
        }
        for (int base_i = 0; base_i < n_surplus; base_i += 32) {
            const int i = base_i + lane;
            bool kept = false;
            float4 pj = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
            if (i < n_surplus) {
                const int j = A.surplus[pos_off + i];
                pj = A.positions32[pos_off + j];
                pj.w = __int_as_float(j);
                ++count;
                kept = keep(pj);
            }
            offer_kept(kept, pj);
        }
        __syncwarp();
        kept_over = buffered > kKeptMax;
        const int solved = kept_over ? kKeptMax : buffered;
        for (int i = lane; i < solved; i += 32) screen_pair(buf[i]);
    }
    float base = fminf(warp_min_float(lane_min_unflagged(key)), t_single);
    int lookups = 0;
    if (far_of<FAR>(ch) == JFGPU_FAR_CELL_BOUNDING) {
        // Far units with the rigorous early rejection -log(1 - u) >= u: a far time is at least
        // u / (beta rate speed), so a unit whose u exceeds reject * rate cannot come before the threshold.  Every far
        // rate of the direction is at most the largest one, so most units are rejected from their keyed draw alone,
        // before anything of theirs is read; only the others read their role word (occupancy cell, or surplus /
        // active) to find their relative cell and rate.
        const float threshold0 = isinf(base) ? kInf32 : base * rel + abs_margin;
        const float reject = threshold0 * speed32 * (1.0f + 1.0f / 65536.0f) / inv_beta32;
        const float largest = sp.far_rate_max32[d];
        if (largest > 0.0f) {
            // u_low = u24 2^-24 > reject * largest  <=>  u24 > cut (u24 an integer; NaN or >= 1: nothing rejected)
            const float scaled = (reject * largest) * 16777216.0f;
            const uint32_t cut = scaled < 16777216.0f ? (uint32_t)scaled : (1u << 24);
            const float *rates = sp.bound_upper32;
            const int32_t *roles = A.roles + pos_off;
            const int16_t *rel_table = A.view.rel + ch.table_offset;
            auto far_unit = [&](int j, uint32_t hi) {
                if ((hi >> 8) > cut || j == active) return;
                ++lookups;
                const int32_t role = roles[j];
                if (role & (kRoleActive | kRoleSurplus)) return;
                const int cx = role & 0xFF, cy = (role >> 8) & 0xFF, cz = (role >> 16) & 0xFF;
                int dx = cx - ax[0], dy = cy - ax[1], dz = cz - ax[2];
                if (dx < 0) dx += m;
                if (dy < 0) dy += m;
                if (dz < 0) dz += m;
                if (((ch.near_mask >> dx) & 1ull) && ((ch.near_mask >> dy) & 1ull) && ((ch.near_mask >> dz) & 1ull))
                    return;
                const int rc = ch.rel_is_mod ? dx + m * (dy + m * dz)
                                             : rel_table[cx * m + ax[0]] +
                                                   m * (rel_table[cy * m + ax[1]] + m * rel_table[cz * m + ax[2]]);
                const float rate = rates[rc * 3 + d];
                if (!(rate > 0.0f)) return;
                const float u_low = (float)(hi >> 8) * (1.0f / 16777216.0f);
                if (u_low > reject * rate) return;
                bool flag = false;
                const float du = expovariate32((uint64_t)hi << 32, inv_beta32, flag);
                float t = (du / rate) / speed32;
                if (flag) t = -1.0f;
                if (!isinf(t)) topk_insert(key, code, t, make_code(j, kPathFar, true));
            };
            // every unit with u24 <= cut is listed when cut < bound: the listed units replace the draws of all n
            const FarAhead &fa = A.ahead[c];
            if (fa.event == (long long)ev && fa.key == ch.key && cut < fa.bound) {
                if (lane < fa.count) far_unit(fa.unit[lane], fa.hi[lane]);
            } else {
                for (int j = lane; j < n; j += 32) far_unit(j, draw_hi32(pair_base, (uint32_t)j));
            }
        }
        base = fminf(base, warp_min_float(lane_min_unflagged(key)));
    }
    const float threshold = isinf(base) ? kInf32 : base * rel + abs_margin;
    // compaction of the candidates inside the threshold into the chain's refine list
    int overflow = (code[kTopK - 1] >= 0 && key[kTopK - 1] <= threshold) ? 1 : 0;
    int total = 0;
#pragma unroll
    for (int i = 0; i < kTopK; ++i) {
        const bool take = code[i] >= 0 && key[i] <= threshold;
        const unsigned mask = __ballot_sync(kFull, take);
        const int offset = total + __popc(mask & ((1u << lane) - 1u));
        if (take && offset < kRefineMax) list.code[offset] = code[i];
        total += __popc(mask);
    }
    overflow = warp_max_int(overflow) || total > A.refine_limit || kept_over;
    const int screened = warp_sum_int(count);
    lookups = warp_sum_int(lookups);
    if (lane == 0) {
        list.count = total < kRefineMax ? total : kRefineMax;
        list.flags = overflow ? kListOverflow : 0;
        list.screened = screened;
        list.far_lookups = lookups;
        if (far_of<FAR>(ch) == JFGPU_FAR_CELL_BOUNDING) A.ahead[c].next = (long long)ev + 1;
    }
    // the entries at the first kRefineSlots offsets go to the queues of their paths, lane q taking entry q
    __syncwarp();
    if (!overflow && lane < kRefineSlots && lane < total) {
        const int path = code_path(list.code[lane]);
        const int at = atomicAdd(queue.counts + (round & 1) * kQueueHalf + path, 1);
        queue.entries[path * queue.stride + at] = (int32_t)(local * kRefineSlots + lane);
    }
}

// One warp per chain: the far units of the chain's next event whose keyed pair draws have u24 < bound (the keyed
// draws of an event depend on nothing that the event before it changes).  Extra blocks of the settle kernel run it,
// beside the round's FP64 re-solves.
__device__ inline void far_ahead_warp(const RunArgs &A, long long local, int lane) {
    if (local >= A.count) return;
    const long long c = A.first_chain + local;
    const ChainDev &ch = A.view.chains[c];
    FarAhead &fa = A.ahead[c];
    const long long next = fa.next;
    if (next < 0 || ch.far != JFGPU_FAR_CELL_BOUNDING || (fa.event == next && fa.key == ch.key)) return;
    const uint64_t base = draw_base(ch.key, (uint64_t)next, kRngPair);
    const uint32_t bound = ahead_bound(ch.n);
    int total = 0;
    for (int j0 = 0; j0 < ch.n; j0 += 32) {
        const int j = j0 + lane;
        uint32_t hi = 0;
        const bool take = j < ch.n && ((hi = draw_hi32(base, (uint32_t)j)) >> 8) < bound;
        const unsigned mask = __ballot_sync(kFull, take);
        const int at = total + __popc(mask & ((1u << lane) - 1u));
        if (take && at < kAhead) {
            fa.unit[at] = j;
            fa.hi[at] = hi;
        }
        total += __popc(mask);
    }
    __syncwarp();
    if (lane == 0) {
        fa.count = total < kAhead ? total : kAhead;
        fa.bound = total <= kAhead ? bound : 0u;
        fa.key = ch.key;
        fa.event = next;
    }
}

struct Refined {
    double q, r, rate;
    int32_t kind, target, aux, status;
};

__device__ inline void load_lifting(const JfgpuChainState &g, const RunArgs &A, const ChainDev &ch, WarpState &w) {
    w.ts_q = g.time_q;
    w.ts_r = g.time_r;
    w.eoc_q = g.eoc_q;
    w.eoc_r = g.eoc_r;
    w.events = g.events;
    w.warnings = g.bound_warnings;
    w.fallbacks = g.refine_fallbacks;
    w.candidates = g.candidates;
    w.refined = g.refined;
    w.lift_sum = g.lift_sum;
    w.liftings = g.liftings;
    w.far_lookups = g.far_lookups;
    w.active = g.active;
    w.direction = g.direction;
    w.eoc_new = g.eoc_new_active;
    w.occ_active = g.occ_active;
    w.occ_cell = g.occ_cell;
    w.n_surplus = g.n_surplus;
    w.status = JFGPU_STATUS_OK;
    w.stop = 0;
    load_pos(A, ch, w.active, w.pa);
}

// every candidate of the event in FP64 by one thread (the rare overflow of a refine list)
template <int POT, int FAR>
__device__ __noinline__ int exact_serial(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                         const WarpState &w, Cand &best) {
    const long long ev = w.events;
    int a[3];
    cell_axes(ch, w.occ_cell, a);
    const int K = ch.n_res;
    const int32_t *occ = A.occupancy + ch.occ_off;
    for (int oz = 0; oz < K; ++oz)
        for (int oy = 0; oy < K; ++oy)
            for (int ox = 0; ox < K; ++ox) {
                const int cell = (a[0] + ch.res[ox]) % ch.m + ch.m * ((a[1] + ch.res[oy]) % ch.m) +
                                 ch.m * ch.m * ((a[2] + ch.res[oz]) % ch.m);
                for (int k = 0; k < ch.max_occ; ++k) {
                    const int j = occ[(long long)cell * ch.max_occ + k];
                    if (j >= 0) JF_TRY(exact_pair_ool<POT>(A, ch, sp, w, j, ev, best));
                }
            }
    for (int i = 0; i < w.n_surplus; ++i)
        JF_TRY(exact_pair_ool<POT>(A, ch, sp, w, A.surplus[ch.pos_off + i], ev, best));
    if (far_of<FAR>(ch) == JFGPU_FAR_CELL_BOUNDING) {
        for (int cell = 0; cell < ch.ncells; ++cell) {
            const int j = occ[cell];
            if (j < 0 || is_nearby(ch, cell, w.occ_cell)) continue;
            JF_TRY(exact_cell_bounding_ool(A, ch, sp, w, j, w.occ_cell, ev, best));
        }
    }
    return JFGPU_STATUS_OK;
}

// A chain's entry in the settle kernel's slots of the round: kRefineSlots FP64 re-solves, then its single candidates
__device__ inline Refined load_refined(const Refined *p) {
    // written by other threads of this kernel: read past L1
    Refined r;
    r.q = __ldcg(&p->q);
    r.r = __ldcg(&p->r);
    r.rate = __ldcg(&p->rate);
    r.kind = __ldcg(&p->kind);
    r.target = __ldcg(&p->target);
    r.aux = __ldcg(&p->aux);
    r.status = __ldcg(&p->status);
    return r;
}

__device__ inline Cand refined_cand(const Refined &rf) {
    Cand cnd;
    cnd.q = rf.q;
    cnd.r = rf.r;
    cnd.kind = rf.kind;
    cnd.target = rf.target;
    cnd.aux = rf.aux;
    cnd.rate = rf.rate;
    return cnd;
}

// The end of a chain's round, by the thread that completes its inputs: the earliest of the single candidates and the
// listed candidates (the FP64 re-solves of the first kRefineSlots entries, the others solved here) is committed and
// the occupancy is updated for the next event.
template <int POT, int FAR>
__device__ inline void settle_chain(const RunArgs &A, const RefineList &list, const Refined *slots, long long c,
                                    long long round) {
    const ChainDev &ch = A.view.chains[c];
    const SpeciesDev &sp = A.view.species[ch.species];
    JfgpuChainState &g = A.state[c];
    WarpState w;
    load_lifting(g, A, ch, w);
    w.candidates += list.screened;
    w.refined += list.count;
    w.far_lookups += list.far_lookups;
    const Refined singles = load_refined(slots + kRefineSlots);
    Cand best = refined_cand(singles);
    int st = singles.status;
    if (!st) {
        // the rare serial re-solves call out of line with a copy of the lifting state, so that the state itself is
        // never addressed and stays in registers
        if (list.flags & kListOverflow) {
            const WarpState frozen = w;
            st = exact_serial<POT, FAR>(A, ch, sp, frozen, best);
            if (potential_of<POT>(ch) != JFGPU_POT_COULOMB) w.fallbacks += 1;
        } else {
            for (int i = 0; i < list.count && i < kRefineSlots && !st; ++i) {
                const Refined rf = load_refined(slots + i);
                if (rf.status) {
                    st = rf.status;
                } else if (rf.kind != (1 << 30)) {
                    const Cand cnd = refined_cand(rf);
                    if (cand_better(cnd, best)) best = cnd;
                }
            }
            if (list.count > kRefineSlots) {
                const WarpState frozen = w;
                for (int i = kRefineSlots; i < list.count && !st; ++i) {
                    const int code = list.code[i];
                    const int j = code_target(code);
                    st = code_far(code)
                             ? exact_cell_bounding_ool(A, ch, sp, frozen, j, frozen.occ_cell, frozen.events, best)
                             : exact_pair_ool<POT>(A, ch, sp, frozen, j, frozen.events, best);
                }
            }
        }
    }
    if (st) {
        w.status = st;
    } else if (A.has_stop && !time_lt(best.q, best.r, A.stop_q, A.stop_r)) {
        time_slice(ch, w, A.stop_q, A.stop_r);
        store_active(A, ch, w, w.active);
        w.stop = 1;
        st = occ_update(A, ch, w);
        if (st) w.status = st;
    } else {
        st = commit(A, ch, sp, w, best, w.occ_cell, c, round);
        if (!st) st = occ_update(A, ch, w);  // the activator's update of the next event
        if (st) w.status = st;
    }
    g.time_q = w.ts_q;
    g.time_r = w.ts_r;
    g.eoc_q = w.eoc_q;
    g.eoc_r = w.eoc_r;
    g.events = w.events;
    g.bound_warnings = w.warnings;
    g.refine_fallbacks = w.fallbacks;
    g.candidates = w.candidates;
    g.refined = w.refined;
    g.lift_sum = w.lift_sum;
    g.liftings = w.liftings;
    g.far_lookups = w.far_lookups;
    g.active = w.active;
    g.direction = w.direction;
    g.eoc_new_active = w.eoc_new;
    g.occ_active = w.occ_active;
    g.occ_cell = w.occ_cell;
    g.n_surplus = w.n_surplus;
    g.status = w.status;
    g.stopped = w.stop;
}

// One of a chain's inputs is in its slot: true for the thread that brings the last one, which settles the chain.
// The count of a chain's inputs is its queued re-solves plus its own thread's single candidates.  Every increment
// releases its thread's slot and the one that completes the count acquires them all; that thread resets the counter
// for the next round.
__device__ inline bool arrive(const RunArgs &A, const RefineList &list, long long c) {
    const int queued = (list.flags & kListOverflow) ? 0 : (list.count < kRefineSlots ? list.count : kRefineSlots);
    int prior;
    // release: this thread's slot is visible before its increment; acquire: the last increment sees every slot
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(prior) : "l"(A.settle + c) : "memory");
    if (prior != queued) return false;
    A.settle[c] = 0;
    return true;
}

// The settle kernel of a round, three kinds of blocks:
//   [0, chain_block)            the FP64 re-solves of the queued entries, one thread each, by screening path: each
//                               path's range is padded to whole warps, so that the 32 threads of a warp re-solve
//                               candidates that take the same branch of the case analysis (up to the rare FP32/FP64
//                               disagreement);
//   [chain_block, ahead_block)  one thread per chain: its single candidates (cell veto, cell boundary, end of chain);
//   [ahead_block, ...)          with the cell-bounding far field, a warp per chain lists the far units' draws of its
//                               next event (far_ahead_warp).
// Each chain settles (settle_chain) as soon as its own inputs are there, not after every chain's re-solves.  The
// queue counters of the round are read here; the other half of the double-buffered counters, which the next
// round's screening fills, is zeroed here.
template <int POT, int FAR>
__global__ void __maxnreg__(128) settle_kernel(RunArgs A, const RefineList *lists, Refined *refined,
                                                                   RefineQueue queue, long long round,
                                                                   int first_round, unsigned chain_block,
                                                                   unsigned ahead_block) {
    if (FAR == JFGPU_FAR_CELL_BOUNDING && blockIdx.x >= ahead_block) {
        const int warps = JF_REFINE_THREADS / 32;
        far_ahead_warp(A, (long long)(blockIdx.x - ahead_block) * warps + (threadIdx.x >> 5), threadIdx.x & 31);
        return;
    }
    long long local;  // the chain of this thread's input
    if (blockIdx.x >= chain_block) {
        local = (long long)(blockIdx.x - chain_block) * blockDim.x + threadIdx.x;
        if (local < kPaths) queue.counts[((round + 1) & 1) * kQueueHalf + local] = 0;
        if (local >= A.count) return;
        const long long c = A.first_chain + local;
        const ChainDev &ch = A.view.chains[c];
        const SpeciesDev &sp = A.view.species[ch.species];
        const JfgpuChainState &g = A.state[c];
        if (g.status != JFGPU_STATUS_OK || (!first_round && g.stopped)) return;
        const RefineList &list = lists[local];
        if (list.flags & kListSkip) return;
        // the listed targets' FP64 positions and role words into L2 for the commit that follows their re-solves
        for (int i = 0; i < list.count && i < kRefineSlots; ++i) {
            const int j = code_target(list.code[i]);
            asm volatile("prefetch.global.L2 [%0];" ::"l"(A.positions + 3 * (ch.pos_off + j)));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(A.roles + ch.pos_off + j));
        }
        WarpState w;
        load_lifting(g, A, ch, w);
        Cand best = cand_none();
        const int st = single_candidates(A, ch, sp, w, w.occ_cell, w.events, best);
        Refined &out = refined[local * (kRefineSlots + 1) + kRefineSlots];
        out.q = best.q;
        out.r = best.r;
        out.rate = best.rate;
        out.kind = best.kind;
        out.target = best.target;
        out.aux = best.aux;
        out.status = st;
    } else {
        const int32_t *counts = queue.counts + (round & 1) * kQueueHalf;
        const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        long long start = 0;
        int path = -1;
        long long index = 0;
#pragma unroll
        for (int k = 0; k < kPaths; ++k) {
            const long long n = counts[k];
            const long long padded = (n + 31) & ~31LL;
            if (path < 0 && t < start + padded) {
                path = k;
                index = t - start;
                if (index >= n) return;
            }
            start += padded;
        }
        if (path < 0) return;
        const int entry = queue.entries[path * queue.stride + index];
        local = entry / kRefineSlots;
        const int slot = entry % kRefineSlots;
        Refined &out = refined[local * (kRefineSlots + 1) + slot];
        const RefineList &list = lists[local];
        const long long c = A.first_chain + local;
        const ChainDev &ch = A.view.chains[c];
        const SpeciesDev &sp = A.view.species[ch.species];
        WarpState w;
        load_lifting(A.state[c], A, ch, w);
        Cand best = cand_none();
        const int code = list.code[slot];
        const int j = code_target(code);
        const int st = code_far(code) ? exact_cell_bounding(A, ch, sp, w, j, w.occ_cell, w.events, best)
                                      : exact_pair<POT>(A, ch, sp, w, j, w.events, best);
        out.q = best.q;
        out.r = best.r;
        out.rate = best.rate;
        out.kind = best.kind;
        out.target = best.target;
        out.aux = best.aux;
        out.status = st;
    }
    const long long c = A.first_chain + local;
    if (arrive(A, lists[local], c))
        settle_chain<POT, FAR>(A, lists[local], refined + local * (kRefineSlots + 1), c, round);
}

#ifndef JF_CHAIN_MIN_BLOCKS
#define JF_CHAIN_MIN_BLOCKS 4
#endif

template <int POT, int FAR>
__global__ void __launch_bounds__(256, JF_CHAIN_MIN_BLOCKS) chains_kernel(RunArgs A) {
    extern __shared__ unsigned char smem_raw[];
    WarpState *shared = reinterpret_cast<WarpState *>(smem_raw);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long local = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
    if (local >= A.count) return;
    const long long c = A.first_chain + local;
    const ChainDev &ch = A.view.chains[c];
    const SpeciesDev &sp = A.view.species[ch.species];
    WarpState &w = shared[warp];
    if (lane == 0) {
        const JfgpuChainState &g = A.state[c];
        w.ts_q = g.time_q;
        w.ts_r = g.time_r;
        w.eoc_q = g.eoc_q;
        w.eoc_r = g.eoc_r;
        w.events = g.events;
        w.warnings = g.bound_warnings;
        w.fallbacks = g.refine_fallbacks;
        w.candidates = g.candidates;
        w.refined = g.refined;
        w.lift_sum = g.lift_sum;
        w.liftings = g.liftings;
        w.active = g.active;
        w.direction = g.direction;
        w.eoc_new = g.eoc_new_active;
        w.occ_active = g.occ_active;
        w.occ_cell = g.occ_cell;
        w.n_surplus = g.n_surplus;
        w.status = g.status;
        w.stop = 0;
        w.real_target = -1;
        load_pos(A, ch, w.active, w.pa);
    }
    __syncwarp();
    const long long start_events = w.events;
    for (long long e = 0; e < A.max_events; ++e) {
        if (w.status != JFGPU_STATUS_OK || w.stop) break;
        if (lane == 0 && w.active != w.occ_active) {
            int st = occ_update_ool(A, ch, w);
            if (st) w.status = st;
        }
        __syncwarp();
        if (w.status != JFGPU_STATUS_OK) break;
        // the active cell of the handlers (position_to_cell of the active position) is the occupancy's
        // active cell just computed from the same position
        const int active_cell = w.occ_cell;
        Cand best;
        int status = JFGPU_STATUS_OK;
        int counted = 0, refined = 0;
        (void)refined;
        status = exact_candidates<POT, FAR>(A, ch, sp, w, active_cell, lane, best, counted);
        __syncwarp();
        if (lane == 0) {
            w.candidates += counted;
            w.refined += refined;
        }
        if (potential_of<POT>(ch) == JFGPU_POT_COULOMB && sp.mic_terms != nullptr && warp_max_int(status) == 0 &&
            !(A.has_stop && !time_lt(best.q, best.r, A.stop_q, A.stop_r))) {
            warp_real_rate(A, ch, sp, w, best, lane);
            __syncwarp();
        }
        if (lane == 0) {
            if (status) {
                w.status = status;
            } else if (A.has_stop && !time_lt(best.q, best.r, A.stop_q, A.stop_r)) {
                time_slice(ch, w, A.stop_q, A.stop_r);
                store_active(A, ch, w, w.active);
                w.stop = 1;
                int st = occ_update_ool(A, ch, w);
                if (st) w.status = st;
            } else {
                int st = commit_ool(A, ch, sp, w, best, active_cell, c, w.events - start_events);
                if (!st) st = occ_update_ool(A, ch, w);  // the activator's update of the next event
                if (st) w.status = st;
            }
            w.real_target = -1;
        }
        __syncwarp();
    }
    if (lane == 0) {
        JfgpuChainState &g = A.state[c];
        g.time_q = w.ts_q;
        g.time_r = w.ts_r;
        g.eoc_q = w.eoc_q;
        g.eoc_r = w.eoc_r;
        g.events = w.events;
        g.bound_warnings = w.warnings;
        g.refine_fallbacks = w.fallbacks;
        g.candidates = w.candidates;
        g.refined = w.refined;
        g.lift_sum = w.lift_sum;
        g.liftings = w.liftings;
        g.active = w.active;
        g.direction = w.direction;
        g.eoc_new_active = w.eoc_new;
        g.occ_active = w.occ_active;
        g.occ_cell = w.occ_cell;
        g.n_surplus = w.n_surplus;
        g.status = w.status;
        g.stopped = w.stop;
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Merged-image Coulomb replicas in the mixed mode, several chains a warp.  Almost every event of these chains is a
// cell-veto event whose work is serial (the alias sample, the potential change, the time arithmetic, the commit):
// FP64 work of one lane, and an FP64 warp instruction occupies GB300's FP64 pipe for 16 cycles however few lanes it
// has.  A group of GW lanes runs each chain, 32 / GW chains a warp, so that one FP64 instruction advances the serial
// step of every chain of the warp.  The single candidates (cell veto, cell boundary, end of chain) come first, in
// FP64 by the group's first lane; their earliest displacement bounds the pair candidates that can still win.  Every
// nearby occupant and surplus unit is screened in FP32 over the group's lanes: the hard core by hs_screen (within
// 2^-12 relative plus the chain's absolute margin unless flagged), the inverse-power Coulomb bound by
// ipcb_x_displacement32 with its rigorous error bound, the potential change in FP32 from the same keyed draw (error
// within 32 units of 2^-24).  A pair whose screened displacement, less its error, does not exceed the bound (or whose
// screen cannot decide) is solved in FP64 with the reference's arithmetic, as the FP64 path solves it; the others
// come after the single candidates and cannot win.  The thinning derivative is shared by the group (mic_x_group,
// equal to the warp's sum bit for bit).
// The events equal the FP64 path's bit for bit.  Groups whose chain has stopped skip the work of an event (their
// lanes are left out of the group's shuffles by masks).
// ---------------------------------------------------------------------------------------------------------------
#ifndef JF_COULOMB_GROUP
#define JF_COULOMB_GROUP 32  // lanes per chain of the grouped Coulomb kernel (8 and 16 measured slower)
#endif

template <int GW>
__device__ inline int group_sum_int(int v, unsigned mask) {
#pragma unroll
    for (int offset = GW / 2; offset > 0; offset >>= 1) v += __shfl_xor_sync(mask, v, offset);
    return v;
}

template <int GW>
__device__ inline int group_max_int(int v, unsigned mask) {
#pragma unroll
    for (int offset = GW / 2; offset > 0; offset >>= 1) v = max(v, __shfl_xor_sync(mask, v, offset));
    return v;
}

template <int GW>
__device__ inline Cand group_argmin(Cand c, unsigned mask) {
#pragma unroll
    for (int offset = GW / 2; offset > 0; offset >>= 1) {
        Cand o;
        o.q = __shfl_xor_sync(mask, c.q, offset);
        o.r = __shfl_xor_sync(mask, c.r, offset);
        o.kind = __shfl_xor_sync(mask, c.kind, offset);
        o.target = __shfl_xor_sync(mask, c.target, offset);
        o.aux = __shfl_xor_sync(mask, c.aux, offset);
        o.rate = __shfl_xor_sync(mask, c.rate, offset);
        if (cand_better(o, c)) c = o;
    }
    return c;
}

// The cell veto's draws of the next GW events of a chain, one event a lane (the Walker sample and the potential
// change keyed by the event index, abstracts/cell_veto_event_handler.py:200-238): they depend on the event, the
// direction and the active unit's charge factor only, so the group's lanes solve them ahead in one pass while
// the chain keeps its direction and charge; the event then takes its lane's relative cell, bounding rate and time
// displacement.  Lane glane holds event w.spec_base + glane.
struct VetoAhead {
    double dt = 0.0, rate = 0.0;
    int rc = 0;
};

template <int GW>
__device__ inline void group_veto_ahead(const ChainDev &ch, const SpeciesDev &sp, WarpState &w, int glane,
                                        int leader, unsigned mask, long long ev, int d, double charge_factor, int which,
                                        VetoAhead &ahead) {
    // the signed factor decides the table (upper or lower bounds) as well as the magnitude
    const double signed_factor = which == 0 ? charge_factor : -charge_factor;
    const bool fresh = w.spec_base >= 0 && ev - w.spec_base < GW && w.spec_d == d && w.spec_factor == signed_factor;
    if (fresh) return;  // uniform over the group: every lane reads the same shared state
    __syncwarp(mask);
    const long long e = ev + glane;
    const WalkerDev &wk = sp.walker[which][d];
    const double total_rate = wk.total_rate * charge_factor;
    const int k = (int)randbelow(draw(ch.key, (uint64_t)e, kRngVetoChoice, 0), (uint32_t)wk.size);
    const double u = wk.mean_rate * uniform53(draw(ch.key, (uint64_t)e, kRngVetoUniform, 0));
    ahead.rc = (u <= wk.first_rate[k]) ? wk.first_item[k] : wk.second_item[k];
    ahead.rate = (which == 0 ? sp.bound_upper[ahead.rc * 3 + d] : sp.bound_lower[ahead.rc * 3 + d]) * charge_factor;
    ahead.dt = expovariate(draw(ch.key, (uint64_t)e, kRngVetoTime, 0), ch.beta) / mul_speed(ch, total_rate);
    __syncwarp(mask);
    if (glane == 0) {
        w.spec_base = ev;
        w.spec_d = d;
        w.spec_factor = signed_factor;
    }
    __syncwarp(mask);
}

// the single candidates of the event (single_candidates with the cell veto solved ahead by the group)
template <int GW>
__device__ inline int group_single_candidates(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                              WarpState &w, int glane, int leader, unsigned mask, long long ev,
                                              VetoAhead &ahead, Cand &best) {
    const int d = w.direction;
    double charge_factor = (charge_of(A, ch, w.active) * 1.0) / 1.0;
    int which = 0;
    if (!(charge_factor > 0.0)) {
        charge_factor *= -1.0;
        which = 1;
    }
    group_veto_ahead<GW>(ch, sp, w, glane, leader, mask, ev, d, charge_factor, which, ahead);
    const int k = (int)(ev - w.spec_base);
    const double dt = __shfl_sync(mask, ahead.dt, leader + k);
    const double rate = __shfl_sync(mask, ahead.rate, leader + k);
    const int rc = __shfl_sync(mask, ahead.rc, leader + k);
    if (glane != 0) return JFGPU_STATUS_OK;
    if (!(rate > 0.0)) return JFGPU_STATUS_ASSERTION;
    const int target_cell = translate_cell(A.view, ch, w.occ_cell, rc);
    offer(best, w.ts_q, w.ts_r, dt, JFGPU_EV_CELL_VETO, -1, target_cell, rate);
    int ax[3];
    cell_axes(ch, w.occ_cell, ax);
    boundary_and_end(A.view, ch, d, ax[d], w.pa[d], w.ts_q, w.ts_r, w.eoc_q, w.eoc_r, w.eoc_new, best);
    return JFGPU_STATUS_OK;
}

// The FP32 screen of a Coulomb pair candidate (the active unit at pa, keyed draws of event ev): false when its event
// provably comes after `bound` (the displacement of the single candidates), true when it must be solved in FP64.
__device__ inline bool coulomb_pair_screen(const RunArgs &A, const ChainDev &ch, const double *pa, long long ev, int d,
                                           double charge_active, float bound, int j) {
    double pj[3], s[3];
    load_pos(A, ch, j, pj);
    separation64(ch, pa, pj, s);
    if (ch.diameter_sq > 0.0) {
        float sv[3] = {(float)s[0], (float)s[1], (float)s[2]};
        bool flag = false;
        const float x = hs_screen(ch.diameter_sq32, d, 1.0f, sv, ch.ulp_margin32, flag);
        if (flag || x * (1.0f - 1.0f / 4096.0f) - ch.screen_abs32 <= bound) return true;
    }
    const uint64_t n = draw(ch.key, (uint64_t)ev, kRngPair, (uint32_t)j) >> 11;
    const float du = n < (1ull << 52) ? -log1pf(-(float)n * 0x1p-53f) * ch.inv_beta32
                                      : -logf((float)((1ull << 53) - n) * 0x1p-53f) * ch.inv_beta32;
    const float du_error = 32.f * 0x1p-24f * du;
    double p[3];
    permute3(s, d, p);
    float error;
    bool unsafe = false;
    const float x = ipcb_x_displacement32((float)(ch.bound_prefactor * charge_active * charge_of(A, ch, j)),
                                          (float)p[0], (float)p[1], (float)p[2], du, du_error, ch.L32, error,
                                          unsafe);
    return unsafe || !(x - error > bound);
}

// the candidates of a chain's event over the GW lanes of its group (mask: the lanes of every group that calls it)
template <int GW>
__device__ inline int group_screened_candidates(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp,
                                                WarpState &w, int glane, int leader, unsigned mask, Cand &best,
                                                int &counted, VetoAhead &ahead) {
    const long long ev = w.events;
    int status = JFGPU_STATUS_OK;
    best = cand_none();
    if (ch.far == JFGPU_FAR_CELL_VETO)
        status = group_single_candidates<GW>(A, ch, sp, w, glane, leader, mask, ev, ahead, best);
    else if (glane == 0)
        status = single_candidates_ool(A, ch, sp, w, w.occ_cell, ev, best);
    double reach = glane == 0 ? time_sub(best.q, best.r, w.ts_q, w.ts_r) * ch.speed : 0.0;
    reach = __shfl_sync(mask, reach, leader);
    const float bound = (float)reach * (1.0f + 1.0f / 1024.0f) + ch.screen_abs32;
    const int d = w.direction;
    const double charge_active = charge_of(A, ch, w.active);
    int count = 0;
    auto screen = [&](int j) {
        ++count;
        if (coulomb_pair_screen(A, ch, w.pa, ev, d, charge_active, bound, j)) {
            const int st = exact_pair_ool<JFGPU_POT_COULOMB>(A, ch, sp, w, j, ev, best);
            if (st) status = st;
        }
    };
    for_each_near(A, ch, w.occ_cell, glane, [&](int j) { screen(j); }, GW);
    for (int i = glane; i < w.n_surplus; i += GW) screen(A.surplus[ch.pos_off + i]);
    counted = group_sum_int<GW>(count, mask);
    best = group_argmin<GW>(best, mask);
    return group_max_int<GW>(status, mask);
}

// warp_real_rate for the group of a chain (mask: the lanes of every group that calls it)
template <int GW>
__device__ inline void group_real_rate(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w,
                                       const Cand &best, int glane, int leader, unsigned mask) {
    int t = -1;
    double pa[3] = {0.0, 0.0, 0.0};
    if (glane == 0) {
        w.real_target = -1;
        if (best.kind == JFGPU_EV_BOUNDED)
            t = best.target;
        else if (best.kind == JFGPU_EV_CELL_VETO)
            t = A.occupancy[ch.occ_off + (long long)best.aux * ch.max_occ];
        if (t >= 0) {
            const double dt = time_sub(best.q, best.r, w.ts_q, w.ts_r);  // as time_slice
            for (int k = 0; k < 3; ++k) pa[k] = w.pa[k];
            pa[w.direction] = py_mod_near(w.pa[w.direction] + ch.speed * dt, ch.L);
        }
    }
    t = __shfl_sync(mask, t, leader);
    const unsigned need = __ballot_sync(mask, t >= 0);
    if (t < 0) return;
    for (int k = 0; k < 3; ++k) pa[k] = __shfl_sync(need, pa[k], leader);
    double pt[3], s[3], p[3];
    load_pos(A, ch, t, pt);
    separation64(ch, pa, pt, s);
    permute3(s, w.direction, p);
    CompositeModel model;
    model.mic = sp.mic;
    model.images = sp.mic_terms;
    model.n_images = sp.mic_images;
    model.rows = sp.mic_terms + sp.mic_images;
    model.n_rows = sp.mic_rows;
    const double scale = mul_speed(ch, ch.coulomb_prefactor * charge_of(A, ch, w.active) * charge_of(A, ch, t));
    if (GW == 32 && best.kind == JFGPU_EV_CELL_VETO && sp.mic_fourier32 != nullptr) {
        // the cell veto's thinning first in FP32: the merged-image sum with its error bound (mic_x_warp32); a
        // rejection (the rate surely below uniform(0, bounding rate), hence also below the bounding rate: no bound
        // warning) is taken here, the real rate stored as 0.0 for the commit's thinning; otherwise the FP64 sum
        model.fourier32 = sp.mic_fourier32;
        model.alpha_over_length32 = (float)sp.mic.alpha_over_length;
        model.alpha_over_length_sq32 = (float)sp.mic.alpha_over_length_sq;
        model.two_alpha_over_length_root_pi32 = (float)sp.mic.two_alpha_over_length_root_pi;
        model.system_length32 = (float)sp.mic.system_length;
        model.two_pi_over_length32 = (float)sp.mic.two_pi_over_length;
        float value32, error32;
        mic_x_warp32(model, (float)p[0], (float)p[1], (float)p[2], glane, value32, error32);
        const double threshold = best.rate * uniform53(draw(ch.key, (uint64_t)w.events, kRngThin, 0));
        const double real_upper = scale * (double)value32 + fabs(scale) * (double)error32 +
                                  fabs(scale * (double)value32) * 0x1p-20;
        if (real_upper < threshold * (1.0 - 0x1p-20)) {
            if (glane == 0) {
                w.real_value = 0.0;
                w.real_target = t;
            }
            return;
        }
    }
    const double value = mic_x_group<GW>(model, p[0], p[1], p[2], glane, need);
    if (glane == 0) {
        w.real_value = mul_speed(ch, ch.coulomb_prefactor * charge_of(A, ch, w.active) * charge_of(A, ch, t) * value);
        w.real_target = t;
    }
}

// 128 registers a thread: the replicas are few warps an SM (1024 chains of a warp each on 152 SMs), so the kernel
// trades occupancy it does not use for fewer spills on its serial FP64 path
constexpr int kRunNear = 64;  // nearby occupants a run of null cell-veto events keeps (more: no run)

// Runs of null cell-veto events (one warp per chain).  Most events of a Coulomb chain with the cell veto move the
// active unit to its veto time and change nothing else: the vetoed cell is empty, the veto comes before the cell
// boundary and the end of chain, and no pair candidate comes before it.  The lanes check the next events of the
// speculation window at once, lane k event ev + k: every lane steps through the time slices of the events before its
// own (the reference's arithmetic, in order), then takes its event's single candidates, its vetoed cell and the FP32
// screen of its pair candidates (an FP64 solve where the screen cannot decide).  The leading events that are null
// are committed together, each exactly as the event loop commits it (time slice, log record, candidate count); the
// first event that is not null is left to the event loop.  Returns the events committed; `broke` tells whether an
// event that is not null ended the run (rather than the window or the event budget).
__device__ inline int warp_null_run(const RunArgs &A, const ChainDev &ch, const SpeciesDev &sp, WarpState &w, int lane,
                                    long long budget, long long log_index, long long chain_index, VetoAhead &ahead,
                                    bool &broke) {
    const long long ev = w.events;
    const int d = w.direction;
    double charge_factor = (charge_of(A, ch, w.active) * 1.0) / 1.0;
    int which = 0;
    if (!(charge_factor > 0.0)) {
        charge_factor *= -1.0;
        which = 1;
    }
#ifndef JF_RUN_REFRESH
#define JF_RUN_REFRESH 16
#endif
    // a window with fewer than 32 - JF_RUN_REFRESH events left is drawn anew from this event, so that a run is not
    // cut short by its end (the draws are pure functions of the event: the same values either way)
    if (lane == 0 && w.spec_base >= 0 && ev - w.spec_base > JF_RUN_REFRESH) w.spec_base = -1;
    __syncwarp();
    group_veto_ahead<32>(ch, sp, w, lane, 0, kFull, ev, d, charge_factor, which, ahead);
    const int k0 = (int)(ev - w.spec_base);  // lane of event ev in the speculation window
    int n_try = 32 - k0;
    if (budget < n_try) n_try = (int)budget;
    broke = false;
    if (n_try < 2) return 0;
    // the vetoed cells do not depend on the time slices: the run ends at the first one that holds a unit (a thinning)
    const int src = k0 + (lane < n_try ? lane : 0);
    const double rate = __shfl_sync(kFull, ahead.rate, src);
    const int rc = __shfl_sync(kFull, ahead.rc, src);
    const int target_cell = translate_cell(A.view, ch, w.occ_cell, rc);
    const bool thinning = lane < n_try && A.occupancy[ch.occ_off + (long long)target_cell * ch.max_occ] >= 0;
    const unsigned thin_mask = __ballot_sync(kFull, thinning);
    if (thin_mask) n_try = __ffs(thin_mask);  // up to and including the first thinning, which fails below
    // the time slices of events ev .. ev + lane, in order (time_add of the veto candidate, then time_slice); every
    // lane steps through all n_try events so that the shuffles stay warp-wide
    double ts_q = w.ts_q, ts_r = w.ts_r, x = w.pa[d];
    double pre_q = 0.0, pre_r = 0.0, pre_x = 0.0, post_q = 0.0, post_r = 0.0, post_x = 0.0, dt_mine = 0.0;
    for (int i = 0; i < n_try; ++i) {
        const double dt = __shfl_sync(kFull, ahead.dt, k0 + i);
        double cq, cr;
        time_add(ts_q, ts_r, dt, cq, cr);
        const double x_next = py_mod_near(x + ch.speed * time_sub(cq, cr, ts_q, ts_r), ch.L);
        if (i == lane) {
            pre_q = ts_q;
            pre_r = ts_r;
            pre_x = x;
            dt_mine = dt;
            post_q = cq;
            post_r = cr;
            post_x = x_next;
        }
        x = x_next;
        ts_q = cq;
        ts_r = cr;
    }
    bool ok = lane < n_try && !thinning && rate > 0.0 && !isinf(dt_mine);
    int count = 0;
    Cand best = cand_none();
    if (ok) {
        int ax[3];
        cell_axes(ch, w.occ_cell, ax);
        // the events before this one left the active unit in its cell (else the occupancy update moves it)
        if (axis_index(A.view, ch, pre_x) != ax[d]) ok = false;
        offer(best, pre_q, pre_r, dt_mine, JFGPU_EV_CELL_VETO, -1, target_cell, rate);
        boundary_and_end(A.view, ch, d, ax[d], pre_x, pre_q, pre_r, w.eoc_q, w.eoc_r, w.eoc_new, best);
        if (best.kind != JFGPU_EV_CELL_VETO || best.q != post_q || best.r != post_r) ok = false;
        if (A.has_stop && !time_lt(post_q, post_r, A.stop_q, A.stop_r)) ok = false;
    }
    // the pair candidates, the same units for every event of the run: the nearby occupants (gathered once by the
    // warp, a cell a lane) and the surplus units
    __shared__ int near_units[8][kRunNear];
    int *units = near_units[threadIdx.x >> 5];
    int n_units = 0;  // warp-uniform
    {
        int a[3];
        cell_axes(ch, w.occ_cell, a);
        const int K = ch.n_res, slots = K * K * K * ch.max_occ;
        const int32_t *occ = A.occupancy + ch.occ_off;
        for (int base = 0; base < slots; base += 32) {
            const int slot = base + lane;
            int j = -1;
            if (slot < slots) {
                const int k = slot / ch.max_occ, ox = k % K, oy = (k / K) % K, oz = k / (K * K);
                int cx = a[0] + ch.res[ox], cy = a[1] + ch.res[oy], cz = a[2] + ch.res[oz];
                if (cx >= ch.m) cx -= ch.m;
                if (cy >= ch.m) cy -= ch.m;
                if (cz >= ch.m) cz -= ch.m;
                j = occ[(long long)(cx + ch.m * (cy + ch.m * cz)) * ch.max_occ + slot % ch.max_occ];
            }
            const unsigned found = __ballot_sync(kFull, j >= 0);
            const int at = n_units + __popc(found & ((1u << lane) - 1u));
            if (j >= 0 && at < kRunNear) units[at] = j;
            n_units += __popc(found);
        }
        __syncwarp();
    }
    if (n_units > kRunNear) ok = false;  // too many to keep: the event loop takes the events one by one
    if (ok) {
        const float bound = (float)(time_sub(post_q, post_r, pre_q, pre_r) * ch.speed) * (1.0f + 1.0f / 1024.0f) +
                            ch.screen_abs32;
        double pa[3] = {w.pa[0], w.pa[1], w.pa[2]};
        pa[d] = pre_x;
        const double charge_active = charge_of(A, ch, w.active);
        auto screen = [&](int j) {
            ++count;
            if (!ok || !coulomb_pair_screen(A, ch, pa, ev + lane, d, charge_active, bound, j)) return;
            WarpState wk = w;  // the state before this lane's event
            wk.pa[d] = pre_x;
            wk.ts_q = pre_q;
            wk.ts_r = pre_r;
            Cand pair = cand_none();
            if (exact_pair_ool<JFGPU_POT_COULOMB>(A, ch, sp, wk, j, ev + lane, pair) || cand_better(pair, best))
                ok = false;
        };
        for (int i = 0; i < n_units; ++i) screen(units[i]);
        for (int i = 0; i < w.n_surplus; ++i) screen(A.surplus[ch.pos_off + i]);
    }
    const unsigned okm = __ballot_sync(kFull, ok);
    const int run = okm == kFull ? 32 : __ffs(~okm) - 1;
    broke = run < n_try;
    if (run == 0) return 0;
    const int counted = warp_sum_int(lane < run ? count : 0);
    if (A.log && lane < run && log_index + lane < A.log_capacity) {
        JfgpuEvent rec;
        rec.kind = JFGPU_EV_CELL_VETO;
        rec.moved = w.active;
        rec.target = -1;
        rec.accepted = 0;
        rec.time_q = post_q;
        rec.time_r = post_r;
        rec.new_active = w.active;
        rec.new_direction = d;
        double p[3] = {w.pa[0], w.pa[1], w.pa[2]};
        p[d] = post_x;
        rec.x = p[0];
        rec.y = p[1];
        rec.z = p[2];
        A.log[(chain_index - A.first_chain) * A.log_capacity + log_index + lane] = rec;
    }
    const double last_q = __shfl_sync(kFull, post_q, run - 1);
    const double last_r = __shfl_sync(kFull, post_r, run - 1);
    const double last_x = __shfl_sync(kFull, post_x, run - 1);
    __syncwarp();
    if (lane == 0) {
        w.ts_q = last_q;
        w.ts_r = last_r;
        w.pa[d] = last_x;
        w.events = ev + run;
        w.candidates += counted;
        store_active(A, ch, w, w.active);
        const int st = occ_update_ool(A, ch, w);  // the activator's update of the next event (the same cell)
        if (st) w.status = st;
    }
    __syncwarp();
    return run;
}

template <int GW>
__global__ void __launch_bounds__(256, 2) coulomb_group_kernel(RunArgs A) {
    constexpr int G = 32 / GW;
    extern __shared__ unsigned char smem_raw[];
    WarpState *shared = reinterpret_cast<WarpState *>(smem_raw);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int group = lane / GW, glane = lane % GW, leader = group * GW;
    const long long local = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * G + group;
    const bool exists = local < A.count;
    if (!__any_sync(kFull, exists)) return;
    const long long c = A.first_chain + (exists ? local : 0);
    const ChainDev &ch = A.view.chains[c];
    const SpeciesDev &sp = A.view.species[ch.species];
    WarpState &w = shared[warp * G + group];
    if (glane == 0 && exists) {
        const JfgpuChainState &g = A.state[c];
        w.ts_q = g.time_q;
        w.ts_r = g.time_r;
        w.eoc_q = g.eoc_q;
        w.eoc_r = g.eoc_r;
        w.events = g.events;
        w.warnings = g.bound_warnings;
        w.fallbacks = g.refine_fallbacks;
        w.candidates = g.candidates;
        w.refined = g.refined;
        w.lift_sum = g.lift_sum;
        w.liftings = g.liftings;
        w.far_lookups = g.far_lookups;
        w.active = g.active;
        w.direction = g.direction;
        w.eoc_new = g.eoc_new_active;
        w.occ_active = g.occ_active;
        w.occ_cell = g.occ_cell;
        w.n_surplus = g.n_surplus;
        w.status = g.status;
        w.stop = 0;
        w.real_target = -1;
        w.spec_base = -1;
        load_pos(A, ch, w.active, w.pa);
    }
    __syncwarp();
    VetoAhead ahead;
    const long long start_events = exists ? w.events : 0;
    long long no_run = -1;  // an event that ended a run of null cell-veto events
    for (long long e = 0; e < A.max_events; ++e) {
        bool live = exists && w.status == JFGPU_STATUS_OK && !w.stop;
        if (!__any_sync(kFull, live)) break;
        if (live && glane == 0 && w.active != w.occ_active) {
            const int st = occ_update_ool(A, ch, w);
            if (st) w.status = st;
        }
        __syncwarp();
        live = live && w.status == JFGPU_STATUS_OK;
        if (GW == 32 && ch.far == JFGPU_FAR_CELL_VETO && live && w.events != no_run) {
            // a run of null cell-veto events, committed together (one chain per warp: live is warp-uniform); the
            // event that ended a run goes through the event loop without a second attempt
            bool broke = false;
            const int run =
                warp_null_run(A, ch, sp, w, lane, A.max_events - e, w.events - start_events, c, ahead, broke);
            if (broke) no_run = w.events;
            if (run > 0) {
                e += run - 1;
                continue;
            }
        }
        const unsigned live_mask = __ballot_sync(kFull, live);
        Cand best = cand_none();
        int status = JFGPU_STATUS_OK, counted = 0;
        if (live)
            status = group_screened_candidates<GW>(A, ch, sp, w, glane, leader, live_mask, best, counted, ahead);
        __syncwarp();
        if (live && glane == 0) w.candidates += counted;
        const bool stop_here = A.has_stop && !time_lt(best.q, best.r, A.stop_q, A.stop_r);
        const bool real = live && status == JFGPU_STATUS_OK && sp.mic_terms != nullptr && !stop_here;
        const unsigned real_mask = __ballot_sync(kFull, real);
        if (real) group_real_rate<GW>(A, ch, sp, w, best, glane, leader, real_mask);
        __syncwarp();
        if (live && glane == 0) {
            if (status) {
                w.status = status;
            } else if (stop_here) {
                time_slice(ch, w, A.stop_q, A.stop_r);
                store_active(A, ch, w, w.active);
                w.stop = 1;
                const int st = occ_update_ool(A, ch, w);
                if (st) w.status = st;
            } else {
                int st = commit_ool(A, ch, sp, w, best, w.occ_cell, c, w.events - start_events);
                if (!st) st = occ_update_ool(A, ch, w);  // the activator's update of the next event
                if (st) w.status = st;
            }
            w.real_target = -1;
        }
        __syncwarp();
    }
    if (exists && glane == 0) {
        JfgpuChainState &g = A.state[c];
        g.time_q = w.ts_q;
        g.time_r = w.ts_r;
        g.eoc_q = w.eoc_q;
        g.eoc_r = w.eoc_r;
        g.events = w.events;
        g.bound_warnings = w.warnings;
        g.refine_fallbacks = w.fallbacks;
        g.candidates = w.candidates;
        g.refined = w.refined;
        g.lift_sum = w.lift_sum;
        g.liftings = w.liftings;
        g.active = w.active;
        g.direction = w.direction;
        g.eoc_new_active = w.eoc_new;
        g.occ_active = w.occ_active;
        g.occ_cell = w.occ_cell;
        g.n_surplus = w.n_surplus;
        g.status = w.status;
        g.stopped = w.stop;
    }
}

// ---------------------------------------------------------------------------------------------------------------
// start of the chains: FP32 mirror, occupancy in particle order (single_active_cell_occupancy.py:95-121),
// lifting state at time 0 (initial_chain_start_of_run_event_handler.py) and the first end-of-chain candidate
// ---------------------------------------------------------------------------------------------------------------
__device__ __noinline__ void init_chain(const EngineView &view, const ChainDev &ch, long long c, double *positions,
                                        float4 *positions32, int32_t *occupancy, int32_t *surplus, int32_t *roles,
                                        float4 *cell_slots, JfgpuChainState *state);

__global__ void init_kernel(EngineView view, long long n_chains, double *positions, float4 *positions32,
                            const double *charges, int32_t *occupancy, int32_t *surplus, int32_t *roles,
                            float4 *cell_slots, JfgpuChainState *state) {
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const long long c = (long long)blockIdx.x * (blockDim.x >> 5) + warp;
    if (c >= n_chains) return;
    const ChainDev &ch = view.chains[c];
    for (int i = lane; i < ch.n; i += 32) {
        const double *p = positions + 3 * (ch.pos_off + i);
        positions32[ch.pos_off + i] =
            make_float4((float)p[0], (float)p[1], (float)p[2], charges ? (float)charges[ch.pos_off + i] : 1.0f);
    }
    for (long long k = lane; k < (long long)ch.ncells * ch.max_occ; k += 32) occupancy[ch.occ_off + k] = -1;
    __syncwarp();
    if (lane == 0) init_chain(view, ch, c, positions, positions32, occupancy, surplus, roles, cell_slots, state);
    __syncwarp();
    // the cell-ordered FP32 mirror of the occupancy just built
    for (long long k = lane; k < (long long)ch.ncells * ch.max_occ; k += 32) {
        const int id = occupancy[ch.occ_off + k];
        const float4 p = id >= 0 ? positions32[ch.pos_off + id] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        cell_slots[ch.occ_off + k] = make_float4(p.x, p.y, p.z, __int_as_float(id));
    }
}

// lane 0 of init_kernel: occupancy in particle order, surplus lists, role words and the chain state
__device__ __noinline__ void init_chain(const EngineView &view, const ChainDev &ch, long long c, double *positions,
                                        float4 *positions32, int32_t *occupancy, int32_t *surplus, int32_t *roles,
                                        float4 *cell_slots, JfgpuChainState *state) {
    int status = JFGPU_STATUS_OK;
    int n_surplus = 0;
    int32_t *occ = occupancy + ch.occ_off;
    for (int i = 0; i < ch.n; ++i) {
        int cell;
        if (cell_of(view, ch, positions + 3 * (ch.pos_off + i), cell)) {
            status = JFGPU_STATUS_CELL_RANGE;
            break;
        }
        int32_t *slots = occ + (long long)cell * ch.max_occ;
        int k = 0;
        while (k < ch.max_occ && slots[k] >= 0) ++k;
        if (k < ch.max_occ) {
            slots[k] = i;
            roles[ch.pos_off + i] = role_of_cell(ch, cell);
        } else {
            roles[ch.pos_off + i] = kRoleSurplus | n_surplus;
            surplus[ch.pos_off + n_surplus++] = i;
        }
    }
    JfgpuChainState g;
    g.time_q = 0.0;
    g.time_r = 0.0;
    time_add(0.0, 0.0, time_sub(0.0, 0.0, 0.0, 0.0) + ch.chain_time, g.eoc_q, g.eoc_r);
    g.events = 0;
    g.bound_warnings = 0;
    g.refine_fallbacks = 0;
    g.candidates = 0;
    g.refined = 0;
    g.active = ch.initial_active;
    g.direction = ch.initial_direction;
    g.eoc_new_active = (int)randbelow(draw(ch.key, 0, kRngNewActive, 0), (uint32_t)ch.n);
    g.occ_active = -1;
    g.occ_cell = -1;
    g.n_surplus = n_surplus;
    g.status = status;
    g.stopped = 0;
    g.lift_sum = 0.0;
    g.liftings = 0;
    g.far_lookups = 0;
    if (status == JFGPU_STATUS_OK) {
        // the activator's first update after the start of the run: the initial active unit leaves the occupancy
        RunArgs A;
        memset(&A, 0, sizeof(A));
        A.view = view;
        A.positions = positions;
        A.positions32 = positions32;
        A.occupancy = occupancy;
        A.surplus = surplus;
        A.roles = roles;
        A.cell_slots = cell_slots;
        WarpState w;
        w.active = g.active;
        w.occ_active = -1;
        w.occ_cell = -1;
        w.n_surplus = n_surplus;
        load_pos(A, ch, w.active, w.pa);
        g.status = occ_update_ool(A, ch, w);
        g.occ_active = w.occ_active;
        g.occ_cell = w.occ_cell;
        g.n_surplus = w.n_surplus;
    }
    state[c] = g;
}

size_t refine_list_bytes() { return sizeof(RefineList); }
size_t far_ahead_bytes() { return sizeof(FarAhead); }
size_t refined_bytes() { return sizeof(Refined) * (kRefineSlots + 1); }
// refine queues of up to 8 chain groups: 32 counters per group, then kPaths slices of n_chains * kRefineSlots entries
size_t refine_queue_bytes(long long n_chains) {
    return sizeof(int32_t) * (8 * 32 + (size_t)kPaths * (size_t)n_chains * kRefineSlots);
}

}  // namespace jf

// ---------------------------------------------------------------------------------------------------------------
// launchers (called by jf_engine_host.cu)
// ---------------------------------------------------------------------------------------------------------------
namespace jf {

// the FP32 mirror (x, y, z, charge) of the FP64 positions of units [first, first + count)
__global__ void mirror_kernel(const double *positions, const double *charges, float4 *positions32, long long first,
                              long long count) {
    const long long i = first + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= first + count) return;
    const double *p = positions + 3 * i;
    positions32[i] = make_float4((float)p[0], (float)p[1], (float)p[2], charges ? (float)charges[i] : 1.0f);
}

// the cell-ordered FP32 mirror of chains [first, first + count) from their occupancy and FP32 mirror, one warp a chain
__global__ void slots_kernel(EngineView view, long long first, long long count, const int32_t *occupancy,
                             const float4 *positions32, float4 *cell_slots) {
    const long long c = first + (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= first + count) return;
    const ChainDev &ch = view.chains[c];
    for (long long k = threadIdx.x & 31; k < (long long)ch.ncells * ch.max_occ; k += 32) {
        const int id = occupancy[ch.occ_off + k];
        const float4 p = id >= 0 ? positions32[ch.pos_off + id] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        cell_slots[ch.occ_off + k] = make_float4(p.x, p.y, p.z, __int_as_float(id));
    }
}

cudaError_t launch_mirror(const EngineView &view, const JfgpuBuffers &b, long long first_chain, long long count,
                          long long first_unit, long long units, cudaStream_t stream) {
    if (units <= 0) return cudaSuccess;
    mirror_kernel<<<(unsigned)((units + 255) / 256), 256, 0, stream>>>(
        b.positions, b.charges, reinterpret_cast<float4 *>(b.positions32), first_unit, units);
    slots_kernel<<<(unsigned)((count + 7) / 8), 256, 0, stream>>>(view, first_chain, count, b.occupancy,
                                                                  reinterpret_cast<const float4 *>(b.positions32),
                                                                  reinterpret_cast<float4 *>(b.cell_slots));
    return cudaGetLastError();
}

cudaError_t launch_init(const EngineView &view, long long n_chains, const JfgpuBuffers &b, const LaunchPlan &plan) {
    const int warps = 4;
    long long blocks = (n_chains + warps - 1) / warps;
    if (plan.clock) plan.clock->begin(plan.stream);
    init_kernel<<<(unsigned)blocks, warps * 32, 0, plan.stream>>>(
        view, n_chains, b.positions, reinterpret_cast<float4 *>(b.positions32), b.charges, b.occupancy, b.surplus,
        b.roles, reinterpret_cast<float4 *>(b.cell_slots), b.state);
    if (plan.clock) plan.clock->end(plan.stream, JFGPU_KERNEL_INIT);
    return cudaGetLastError();
}

// one group of chains [A.first_chain, A.first_chain + A.count) with its slices of the refine lists
struct GroupLaunch {
    RunArgs args;
    RefineList *lists;
    Refined *refined;
    RefineQueue queue;
    cudaStream_t stream;
};

// Rounds [r0, r0 + n) of the mixed mode: per round the screening and the settle kernel of every group, issued round
// by round so that the groups' streams advance together; `clock` (may be null) brackets the rounds it samples.  The
// round index reaches the kernels for the event log and the parity of the queue counters; `first_round` marks round
// 0 of a run call, where chains stopped by an earlier call start again.
template <int POT, int FAR>
static long long issue_rounds(const GroupLaunch *groups, int n_groups, long long r0, long long n, int warps,
                              KernelClock *clock) {
    long long launches = 0;
    for (long long r = r0; r < r0 + n; ++r) {
        KernelClock *timed = (clock && r % clock->stride == 0) ? clock : nullptr;
        const int first_round = r == 0 ? 1 : 0;
        for (int g = 0; g < n_groups; ++g) {
            const GroupLaunch &G = groups[g];
            if (timed) timed->begin(G.stream);
            const long long count = G.args.count;
            const long long screen_blocks = (count + warps - 1) / warps;
            // settle blocks: every queued entry plus the padding of each path to whole warps, a thread per chain, and
            // with the cell-bounding far field a warp per chain for the far units' draws of its next event
            const long long refine_blocks =
                (count * kRefineSlots + kPaths * 31 + JF_REFINE_THREADS - 1) / JF_REFINE_THREADS;
            const long long chain_blocks = (count + JF_REFINE_THREADS - 1) / JF_REFINE_THREADS;
            const long long ahead_blocks =
                FAR == JFGPU_FAR_CELL_BOUNDING ? (count + JF_REFINE_THREADS / 32 - 1) / (JF_REFINE_THREADS / 32) : 0;
            screen_kernel<POT, FAR><<<(unsigned)screen_blocks, warps * 32, warps * kKeptMax * sizeof(float4),
                                      G.stream>>>(G.args, G.lists, G.queue, r, first_round);
            if (timed) timed->end(G.stream, JFGPU_KERNEL_SCREEN);
            settle_kernel<POT, FAR>
                <<<(unsigned)(refine_blocks + chain_blocks + ahead_blocks), JF_REFINE_THREADS, 0, G.stream>>>(
                    G.args, G.lists, G.refined, G.queue, r, first_round, (unsigned)refine_blocks,
                    (unsigned)(refine_blocks + chain_blocks));
            if (timed) timed->end(G.stream, JFGPU_KERNEL_RESOLVE);
            launches += 2;
        }
    }
    return launches;
}

// Captured round segments, replayed with one graph launch: the per-launch costs of the three kernels per round and
// group shrink to those of a graph node.  A segment is keyed by everything its launches bake in.
struct SegmentKey {
    RunArgs args;
    void *lists, *refined, *queue;
    long long rounds;
    int first, warps, groups, pot, far;
    bool operator<(const SegmentKey &o) const { return memcmp(this, &o, sizeof(SegmentKey)) < 0; }
};

class GraphCache {
  public:
    ~GraphCache() {
        for (auto &entry : graphs_) cudaGraphExecDestroy(entry.second);
        if (stream) cudaStreamDestroy(stream);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
    }
    // the stream the segments are captured on and replayed on, and the events that order it after and before the
    // caller's stream (created on first use, on the current device)
    bool ready() {
        if (stream) return true;
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return true;
    }
    cudaGraphExec_t find(const SegmentKey &key) {
        auto it = graphs_.find(key);
        return it == graphs_.end() ? nullptr : it->second;
    }
    void insert(const SegmentKey &key, cudaGraphExec_t exec) {
        if (graphs_.size() >= kMaxGraphs) {  // a batch reuses few shapes; a full cache starts afresh
            for (auto &entry : graphs_) cudaGraphExecDestroy(entry.second);
            graphs_.clear();
        }
        graphs_[key] = exec;
    }
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

  private:
    static constexpr size_t kMaxGraphs = 32;
    std::map<SegmentKey, cudaGraphExec_t> graphs_;
};

void *graph_cache_create() { return new GraphCache(); }
void graph_cache_destroy(void *cache) { delete static_cast<GraphCache *>(cache); }

// rounds [r0, r0 + n) of one chain group as one graph on the cache's stream, ordered after the caller's stream and
// before its next work: captured the first time this segment is met, replayed afterwards
template <int POT, int FAR>
static long long replay_rounds(const GroupLaunch &group, long long r0, long long n, int warps, const LaunchPlan &plan,
                               GraphCache *cache, SegmentKey key) {
    key.rounds = n;
    key.first = (r0 == 0 ? 1 : 0) | (int)((r0 & 1) << 1);  // the first round, and the parity of the queue counters
    GroupLaunch G = group;
    G.stream = cache->stream;
    cudaGraphExec_t exec = cache->find(key);
    if (!exec) {
        if (cudaStreamBeginCapture(cache->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return issue_rounds<POT, FAR>(&group, 1, r0, n, warps, nullptr);
        }
        issue_rounds<POT, FAR>(&G, 1, r0, n, warps, nullptr);
        cudaGraph_t graph = nullptr;
        if (cudaStreamEndCapture(cache->stream, &graph) != cudaSuccess || !graph) {
            cudaGetLastError();
            return issue_rounds<POT, FAR>(&group, 1, r0, n, warps, nullptr);
        }
        const cudaError_t made = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (made != cudaSuccess) {
            cudaGetLastError();
            return issue_rounds<POT, FAR>(&group, 1, r0, n, warps, nullptr);
        }
        cache->insert(key, exec);
    }
    cudaEventRecord(cache->fork, group.stream);
    cudaStreamWaitEvent(cache->stream, cache->fork, 0);
    cudaGraphLaunch(exec, cache->stream);
    cudaEventRecord(cache->join, cache->stream);
    cudaStreamWaitEvent(group.stream, cache->join, 0);
    return 2 * n;
}

// All rounds of a run call.  One chain group without an event log: graph segments (with timing on, every sampled
// round is launched plainly between graphs of the rounds in between); otherwise, or when the caller's stream is
// itself being captured, plain launches.
template <int POT, int FAR>
static long long launch_mixed_rounds(const GroupLaunch *groups, int n_groups, long long rounds, int warps,
                                     const LaunchPlan &plan, bool graphs, const SegmentKey &key) {
    GraphCache *cache = static_cast<GraphCache *>(plan.graphs);
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    if (graphs && (cudaStreamIsCapturing(groups[0].stream, &capturing) != cudaSuccess ||
                   capturing != cudaStreamCaptureStatusNone)) {
        cudaGetLastError();
        graphs = false;
    }
    if (!graphs || !cache || n_groups != 1 || !cache->ready())
        return issue_rounds<POT, FAR>(groups, n_groups, 0, rounds, warps, plan.clock);
    if (!plan.clock) return replay_rounds<POT, FAR>(groups[0], 0, rounds, warps, plan, cache, key);
    long long launches = 0;
    const long long stride = plan.clock->stride;
    for (long long r = 0; r < rounds; r += stride) {
        launches += issue_rounds<POT, FAR>(groups, 1, r, 1, warps, plan.clock);  // the sampled round
        const long long n = (r + stride < rounds ? r + stride : rounds) - (r + 1);
        if (n > 0) launches += replay_rounds<POT, FAR>(groups[0], r + 1, n, warps, plan, cache, key);
    }
    return launches;
}

cudaError_t launch_run(const EngineView &view, const JfgpuBuffers &b, long long first, long long count,
                       long long max_events, double stop_q, double stop_r, int mode, JfgpuEvent *log,
                       long long log_capacity, int uniform_potential, int uniform_far, void *lists, void *refined,
                       void *queue, void *ahead, void *settle, long long n_chains, const LaunchPlan &plan,
                       long long *launches) {
    RunArgs A;
    memset(&A, 0, sizeof(A));  // padding included: the arguments key the graph cache bytewise
    A.view = view;
    A.positions = b.positions;
    A.positions32 = reinterpret_cast<float4 *>(b.positions32);
    A.charges = b.charges;
    A.occupancy = b.occupancy;
    A.surplus = b.surplus;
    A.roles = b.roles;
    A.cell_slots = reinterpret_cast<float4 *>(b.cell_slots);
    A.state = b.state;
    A.log = log;
    A.log_capacity = log_capacity;
    A.first_chain = first;
    A.count = count;
    A.max_events = max_events;
    A.stop_q = stop_q;
    A.stop_r = stop_r;
    A.has_stop = isinf(stop_q) ? 0 : 1;
    A.refine_limit = plan.refine_limit < 1 ? 1 : (plan.refine_limit > kRefineMax ? kRefineMax : plan.refine_limit);
    A.ahead = static_cast<FarAhead *>(ahead);
    A.settle = static_cast<int32_t *>(settle);
    int warps = plan.warps;
    if (warps < 1) warps = 1;
    if (warps > 8) warps = 8;
    if (count < warps) warps = (int)count;
    // merged-image Coulomb chains (a few dozen charges, almost every event a cell-veto event) run the warp-per-chain
    // kernel in either mode: the mixed mode screens their pair candidates in FP32 (screened_candidates)
    const bool coulomb_screen = mode == JFGPU_MODE_MIXED && uniform_potential == JFGPU_POT_COULOMB &&
                                uniform_far == JFGPU_FAR_CELL_VETO;
    if (mode == JFGPU_MODE_MIXED && uniform_potential == JFGPU_POT_COULOMB) mode = JFGPU_MODE_EXACT;
    if (mode == JFGPU_MODE_MIXED) {
        // groups of at least one block of warps each; the event log stays on the caller's stream
        int n_groups = plan.groups;
        if (log || !plan.group_streams) n_groups = 1;
        if (n_groups > 8) n_groups = 8;
        while (n_groups > 1 && count < (long long)n_groups * 32) --n_groups;
        GroupLaunch groups[8];
        const long long chunk = (count + n_groups - 1) / n_groups;
        int used = 0;
        for (int g = 0; g < n_groups; ++g) {
            const long long lo = g * chunk, hi = count < lo + chunk ? count : lo + chunk;
            if (hi <= lo) break;
            GroupLaunch &G = groups[used++];
            G.args = A;
            G.args.first_chain = first + lo;
            G.args.count = hi - lo;
            G.args.log = nullptr;
            G.lists = static_cast<RefineList *>(lists) + lo;
            G.refined = static_cast<Refined *>(refined) + lo * (kRefineSlots + 1);
            G.queue.counts = static_cast<int32_t *>(queue) + 32 * g;
            G.queue.entries = static_cast<int32_t *>(queue) + 8 * 32 + (first + lo) * kRefineSlots;
            G.queue.stride = n_chains * kRefineSlots;
            G.stream = n_groups > 1 ? plan.group_streams[g] : plan.stream;
        }
        // counters start at zero in every run (a run that stopped on an error may have left some behind)
        cudaMemsetAsync(queue, 0, sizeof(int32_t) * 8 * 32, plan.stream);
        if (n_groups == 1) groups[0].args.log = log;
        if (used > 1) {
            cudaEventRecord(plan.fork, plan.stream);
            for (int g = 0; g < used; ++g) cudaStreamWaitEvent(groups[g].stream, plan.fork, 0);
        }
        SegmentKey key;
        memset(&key, 0, sizeof(key));
        key.args = A;
        key.lists = lists;
        key.refined = refined;
        key.queue = queue;
        key.warps = warps;
        key.groups = used;
        key.pot = uniform_potential;
        key.far = uniform_far;
        const bool graphs = plan.graphs != nullptr && log == nullptr;
        // kernels specialised for the common homogeneous batches carry only their potential's code
        long long issued;
        if (uniform_potential == JFGPU_POT_LENNARD_JONES && uniform_far == JFGPU_FAR_CELL_BOUNDING)
            issued = launch_mixed_rounds<JFGPU_POT_LENNARD_JONES, JFGPU_FAR_CELL_BOUNDING>(groups, used, max_events,
                                                                                          warps, plan, graphs, key);
        else if (uniform_potential == JFGPU_POT_LENNARD_JONES && uniform_far == JFGPU_FAR_CELL_VETO)
            issued = launch_mixed_rounds<JFGPU_POT_LENNARD_JONES, JFGPU_FAR_CELL_VETO>(groups, used, max_events, warps,
                                                                                      plan, graphs, key);
        else if (uniform_potential == JFGPU_POT_HARD_SPHERE && uniform_far == JFGPU_FAR_NONE)
            issued = launch_mixed_rounds<JFGPU_POT_HARD_SPHERE, JFGPU_FAR_NONE>(groups, used, max_events, warps,
                                                                               plan, graphs, key);
        else
            issued = launch_mixed_rounds<-1, -1>(groups, used, max_events, warps, plan, graphs, key);
        if (used > 1) {
            for (int g = 0; g < used; ++g) {
                cudaEventRecord(plan.join[g], groups[g].stream);
                cudaStreamWaitEvent(plan.stream, plan.join[g], 0);
            }
        }
        *launches += issued;
    } else {
        const long long blocks = (count + warps - 1) / warps;
        const size_t smem = sizeof(WarpState) * warps;
        if (plan.clock) plan.clock->begin(plan.stream);
        if (coulomb_screen) {
            constexpr int G = 32 / JF_COULOMB_GROUP;
            const long long group_blocks = (count + (long long)warps * G - 1) / ((long long)warps * G);
            coulomb_group_kernel<JF_COULOMB_GROUP>
                <<<(unsigned)group_blocks, warps * 32, smem * G, plan.stream>>>(A);
        } else {
            chains_kernel<-1, -1><<<(unsigned)blocks, warps * 32, smem, plan.stream>>>(A);
        }
        if (plan.clock) plan.clock->end(plan.stream, JFGPU_KERNEL_CHAINS);
        *launches += 1;
    }
    return cudaGetLastError();
}

}  // namespace jf
