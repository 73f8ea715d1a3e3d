/*
 * jfgpu.h -- C ABI of the GB300 event-time engine for event-chain Monte Carlo (libjfgpu.so).
 *
 * Plain pointers and sizes only.  Arrays named "device" live in GPU memory owned by the caller (for example
 * PyTorch tensors); the library owns only engines (contexts) and the lookup tables inside them.  Every function
 * returns JFGPU_OK (0) or a nonzero error code and never aborts; per-element and per-chain results carry the
 * status codes of the reference's exceptions (JFGPU_STATUS_*).  Streams are cudaStream_t passed as void*
 * (NULL = the legacy default stream).
 *
 * Reference interfaces replaced (paths relative to the JeLLyFysh source tree):
 *   jfgpu_*_displacement / jfgpu_*_derivative
 *       Potential.displacement / Potential.derivative          jellyfysh/potential/potential.py:153-253
 *       (hard_sphere_potential.py:65-99, inverse_power_potential.py:71-179, lennard_jones_potential.py:63-135,
 *        displaced_even_power_potential.py:73-142, abstracts.py:212-530,
 *        inverse_power_coulomb_bounding_potential.c:53-139 via .py:111-140,
 *        merged_image_coulomb_potential.c:205-274 via .py:128-154, cell_bounding_potential.py:155-238)
 *   jfgpu_engine_create
 *       construct_* / destroy_* contexts                        merged_image_coulomb_potential.c:77-156
 *       CellBoundingPotential.initialize, CellVetoEventHandler.initialize (estimator scans, Walker tables)
 *                                                               cell_bounding_potential.py:70-126,
 *                                                               cell_veto_event_handler.py:93-160, walker.py:53-103
 *   jfgpu_chains_init / jfgpu_chains_run
 *       SingleProcessMediator.run with the event handlers, the heap scheduler, the tree state handler and the
 *       single-active cell occupancy of the path              jellyfysh/mediator/single_process_mediator.py:91-156,
 *       two_leaf_unit_event_handler.py:98-154, two_leaf_unit_bounding_potential_event_handler.py:112-168,
 *       two_leaf_unit_cell_bounding_potential_event_handler.py:137-211, cell_veto_event_handler.py:162-238,
 *       leaf_unit_cell_veto_event_handler.py:117-149, cell_boundary_event_handler.py:98-173,
 *       single_independent_active_periodic_direction_end_of_chain_event_handler.py:151-237,
 *       scheduler/heap_scheduler/heap.c:156-304, activator/internal_state/single_active_cell_occupancy.py:95-237
 *   jfgpu_water_run / jfgpu_water_cells_run
 *       SingleProcessMediator.run over flexible water: factor-type-map bonds and Lennard-Jones,
 *       two_composite_object_summed_bounding_potential_event_handler.py:119-202, lifting/lifting.py:47-108;
 *       with molecular cells the reference's water cell-veto configuration
 *       (config_files/2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini): root units in
 *       single_active_cell_occupancy.py:95-203, composite_object_cell_veto_event_handler.py:110-162,
 *       cell_boundary_event_handler.py:98-173, excluded_cells_tagger.py:107-132, surplus_cells_tagger.py:107-131
 */
#ifndef JFGPU_H
#define JFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---- */
#define JFGPU_OK 0
#define JFGPU_ERROR_CUDA 1
#define JFGPU_ERROR_ARGUMENT 2
#define JFGPU_ERROR_ALLOCATION 3
#define JFGPU_ERROR_TABLE 4

/* ---- per-element / per-chain status (the reference's exceptions) ---- */
#define JFGPU_STATUS_OK 0
#define JFGPU_STATUS_VALUE_ERROR 1     /* math.sqrt of a negative number */
#define JFGPU_STATUS_ASSERTION 2       /* a failed assert of the reference */
#define JFGPU_STATUS_ZERO_DIVISION 3   /* ZeroDivisionError of a float division */
#define JFGPU_STATUS_COMPLEX 4         /* negative ** fractional */
#define JFGPU_STATUS_CELL_RANGE 7      /* position outside the cell list */
#define JFGPU_STATUS_EVENT_CAP 8       /* the refinement set of a mixed-precision event overflowed twice */
#define JFGPU_STATUS_LIFTING 9         /* LiftingSchemeError: the lifting table holds no active unit */
#define JFGPU_STATUS_INDEX 10          /* IndexError: the lifting table holds no negative derivative */

/* ---- potentials ---- */
#define JFGPU_POT_HARD_SPHERE 0
#define JFGPU_POT_LENNARD_JONES 1
#define JFGPU_POT_COULOMB 2            /* merged-image Coulomb bounded by the inverse-power Coulomb bound */

/* ---- far fields ---- */
#define JFGPU_FAR_NONE 0
#define JFGPU_FAR_CELL_VETO 1
#define JFGPU_FAR_CELL_BOUNDING 2

/* ---- run modes ---- */
#define JFGPU_MODE_EXACT 0             /* every candidate solved in FP64 with the reference's arithmetic */
#define JFGPU_MODE_MIXED 1             /* FP32 screening of all candidates, FP64 re-solve of the near-winners */

/* ---- event kinds of the event log ---- */
#define JFGPU_EV_PAIR 0
#define JFGPU_EV_BOUNDED 1
#define JFGPU_EV_HARDCORE 2
#define JFGPU_EV_CELL_BOUNDING 3
#define JFGPU_EV_CELL_VETO 4
#define JFGPU_EV_BOUNDARY 5
#define JFGPU_EV_END_OF_CHAIN 6
#define JFGPU_EV_BOND 8                /* intramolecular bond of a water molecule (lifting) */
#define JFGPU_EV_COMPOSITE 9           /* Coulomb factor of two molecules (thinning, lifting within both) */

/* ======================================================================================================
 * Potentials: batched displacement / derivative.  velocity and separation are device arrays [n][3];
 * charges are device arrays [n][2] (charge of the active unit, charge of the target unit);
 * potential_change is a device array [n]; out [n] receives the time displacement (inf = no event) or the
 * time derivative; status [n] receives JFGPU_STATUS_* per element.
 * ==================================================================================================== */
int jfgpu_hard_sphere_displacement(double radius, const double *velocity, const double *separation, int64_t n,
                                   double *out, int32_t *status, void *stream);
int jfgpu_inverse_power_displacement(double power, double prefactor, const double *velocity,
                                     const double *separation, const double *charges,
                                     const double *potential_change, int64_t n, double *out, int32_t *status,
                                     void *stream);
int jfgpu_inverse_power_derivative(double power, double prefactor, const double *velocity, const double *separation,
                                   const double *charges, int64_t n, double *out, int32_t *status, void *stream);
int jfgpu_lennard_jones_displacement(double prefactor, double characteristic_length, const double *velocity,
                                     const double *separation, const double *potential_change, int64_t n,
                                     double *out, int32_t *status, void *stream);
int jfgpu_lennard_jones_derivative(double prefactor, double characteristic_length, const double *velocity,
                                   const double *separation, int64_t n, double *out, int32_t *status,
                                   void *stream);
int jfgpu_displaced_even_power_displacement(double equilibrium_separation, int32_t power, double prefactor,
                                            const double *velocity, const double *separation,
                                            const double *potential_change, int64_t n, double *out,
                                            int32_t *status, void *stream);
int jfgpu_displaced_even_power_derivative(double equilibrium_separation, int32_t power, double prefactor,
                                          const double *velocity, const double *separation, int64_t n,
                                          double *out, int32_t *status, void *stream);
int jfgpu_coulomb_bound_displacement(double prefactor, double system_length, const double *velocity,
                                     const double *separation, const double *charges,
                                     const double *potential_change, int64_t n, double *out, int32_t *status,
                                     void *stream);
int jfgpu_coulomb_bound_derivative(double prefactor, const double *velocity, const double *separation,
                                   const double *charges, int64_t n, double *out, int32_t *status, void *stream);
int jfgpu_merged_image_coulomb_derivative(double alpha, int32_t fourier_cutoff, int32_t position_cutoff,
                                          double prefactor, double system_length, const double *velocity,
                                          const double *separation, const double *charges, int64_t n,
                                          double *out, int32_t *status, void *stream);
/* The same derivative for callers that cannot allocate device memory (no counterpart in the reference, whose
 * C extension keeps its table in host memory).  jfgpu_merged_image_coulomb_derivative allocates its
 * Fourier-coefficient table on every call; hosts that must not enter the CUDA allocator while running (real-time
 * loops, a fixed memory budget) and plug-ins inside another framework's memory pool cannot.  This entry point keeps
 * the table in a fixed file-scope device array (32 KiB, held by every GPU that loads the library until the process
 * exits), fills it on the device from the parameters passed by value, and calls no allocation routine.  Limit:
 * fourier_cutoff <= 15, larger values return JFGPU_ERROR_ARGUMENT.  Its first call on a device looks up the array's
 * device address with that device current.  Every call shares the
 * array and rewrites it: calls that overlap on the GPU (different streams without ordering) race. */
int jfgpu_merged_image_coulomb_derivative_noalloc(double alpha, int32_t fourier_cutoff, int32_t position_cutoff,
                                                  double prefactor, double system_length, const double *velocity,
                                                  const double *separation, const double *charges, int64_t n,
                                                  double *out, int32_t *status, void *stream);
/* CellBoundingPotential.displacement: potential_change / rate, rate = bounds[cell_separation][direction]
 * (times the charge correction factor; the lower bound when that factor is not positive). bounds_upper and
 * bounds_lower are device arrays [cells][3]; cell_separation, direction device arrays [n]; charge_factor [n]. */
int jfgpu_cell_bounding_displacement(const double *bounds_upper, const double *bounds_lower,
                                     const int32_t *cell_separation, const int32_t *direction, const double *speed,
                                     const double *charge_factor, const double *potential_change, int64_t n,
                                     double *out, int32_t *status, void *stream);

/* ======================================================================================================
 * Lifting schemes of composite objects: the new active unit after an event between more than two units.
 * Replaces Lifting.reset / insert / get_active_identifier (jellyfysh/lifting/lifting.py:47-108) of
 * InsideFirstLifting (lifting/inside_first_lifting.py:37-54), OutsideFirstLifting
 * (lifting/outside_first_lifting.py:38-55) and RatioLifting (lifting/ratio_lifting.py:38-56), as the event
 * handlers of composite objects fill and query them (event_handler/abstracts/
 * event_handler_with_bounding_potential.py:170-220).
 * ==================================================================================================== */
#define JFGPU_LIFTING_INSIDE_FIRST 0
#define JFGPU_LIFTING_OUTSIDE_FIRST 1
#define JFGPU_LIFTING_RATIO 2
#define JFGPU_DRAW_VALUE 0             /* draws[i] is the value random.uniform(0.0, b) returned */
#define JFGPU_DRAW_UNIT 1              /* draws[i] is random(), the value is 0.0 + (b - 0.0) * draws[i] */
/* n tables in one launch.  Table i is entries offsets[i] .. offsets[i+1]-1 of rates (the factor derivatives in
 * insertion order) and active (1 for the active unit); offsets is a device array [n+1], non-decreasing.
 * draws[i] decides table i: the draw of the active unit's insert for inside-first and outside-first, the draw of
 * get_active_identifier for ratio.  selected[i] receives the index within table i of the new active unit (-1
 * on an error), bound[i] the upper end b of that random.uniform(0.0, b) call (NaN when the reference raises
 * before it), status[i] JFGPU_STATUS_OK, _ASSERTION (an active unit with a derivative <= 0, or a second
 * active unit), _LIFTING (no active unit) or _INDEX (no negative derivative).  bound may be null; with n = 0
 * every pointer may be null. */
int jfgpu_lifting(int32_t scheme, int32_t draw_mode, const double *rates, const int32_t *active,
                  const int64_t *offsets, int64_t n, const double *draws, int64_t *selected, double *bound,
                  int32_t *status, void *stream);

/* ======================================================================================================
 * Composite objects: events between two composite objects (dipoles, water molecules) of `units` point charges
 * each, merged-image Coulomb between the charges, bounded pair by pair by the inverse-power Coulomb bound and
 * summed over the target object.  Replaces TwoCompositeObjectSummedBoundingPotentialEventHandler
 * (event_handler/two_composite_object_summed_bounding_potential_event_handler.py:119-202) with its
 * _fill_lifting (event_handler/abstracts/event_handler_with_bounding_potential.py:170-220) and lifting scheme.
 * Position arrays are device arrays of 3 doubles per unit; unit arrays of an event are contiguous.
 * ==================================================================================================== */
typedef struct {
    int32_t units;                /* leaf units per composite object, 1..8 */
    int32_t lifting;              /* JFGPU_LIFTING_* */
    int32_t fourier_cutoff;       /* MergedImageCoulombPotential */
    int32_t position_cutoff;
    double alpha;
    double coulomb_prefactor;
    double bound_prefactor;       /* InversePowerCoulombBoundingPotential */
    double system_length;
} JfgpuCompositeDesc;
/* send_event_time (:119-150) of n events: displacement[i] = min over the target units j of the bounding
 * displacement of the active unit (velocity [n][3], active_position [n][3], active_charge [n]) against target unit
 * j (target_positions [n][units][3], target_charges [n][units]) with potential change potential_changes[i][j] (the
 * reference's random.expovariate(beta) per target unit, in target order). */
int jfgpu_composite_event_time(const JfgpuCompositeDesc *desc, const double *velocity, const double *active_position,
                               const double *active_charge, const double *target_positions,
                               const double *target_charges, const double *potential_changes, int64_t n,
                               double *displacement, int32_t *status, void *stream);
/* send_out_state (:152-202) of n events at the event time.  local_positions / target_positions [n][units][3] and
 * charges [n][units], each object's units sorted by identifier; active_index [n] the active unit among the local
 * ones; local_first [n] 1 when the local object's identifier is the smaller (the derivative table lists it
 * first).  draws [n][3]: the thinning draw random.uniform(0.0, bounding rate), the draw of the active unit's
 * insert into the lifting table, the ratio scheme's draw of get_active_identifier (unused by the other schemes);
 * draw_mode JFGPU_DRAW_VALUE or JFGPU_DRAW_UNIT as for jfgpu_lifting.  new_active [n]: -1 when the event is
 * thinned out, i for local unit i, units + j for target unit j.  rates [n][2] (may be null): the summed bounding
 * event rate and the event rate max(0, factor derivative).  status [n]: JFGPU_STATUS_* (lifting statuses as for
 * jfgpu_lifting; _ASSERTION for a velocity that is not along one positive axis). */
int jfgpu_composite_out_state(const JfgpuCompositeDesc *desc, int32_t draw_mode, const double *velocity,
                              const double *local_positions, const double *local_charges,
                              const int32_t *active_index, const double *target_positions,
                              const double *target_charges, const int32_t *local_first, const double *draws,
                              int64_t n, int32_t *new_active, double *rates, int32_t *status, void *stream);

/* Molecular cell-bounding and cell-veto handlers (the far field between composite objects):
 * TwoCompositeObjectCellBoundingPotentialEventHandler (two_composite_object_cell_bounding_potential_event_handler.py:
 * 153-265) and CompositeObjectCellVetoEventHandler (composite_object_cell_veto_event_handler.py:110-162 with
 * abstracts/cell_veto_event_handler.py:162-238).  Their out-state is send_out_state of the summed handler with the
 * thinning drawn against a given bounding event rate: jfgpu_composite_bounded_out_state takes bounding_rates [n]
 * (the cell-bounding rate times the speed, or the cell veto's rate) and otherwise the arguments and outputs of
 * jfgpu_composite_out_state (rates [n][2] returns the given rate and the event rate; desc->bound_prefactor is
 * unused). */
int jfgpu_composite_bounded_out_state(const JfgpuCompositeDesc *desc, int32_t draw_mode, const double *velocity,
                                      const double *local_positions, const double *local_charges,
                                      const int32_t *active_index, const double *target_positions,
                                      const double *target_charges, const int32_t *local_first,
                                      const double *bounding_rates, const double *draws, int64_t n,
                                      int32_t *new_active, double *rates, int32_t *status, void *stream);
/* The cell-bounding event time of n events: CellBoundingPotential.standard_velocity_displacement
 * (cell_bounding_potential.py:155-198) through Potential.displacement, with DipoleMonteCarloEstimator's charge factor
 * (estimator/dipole_monte_carlo_estimator.py:157-190).  upper / lower [cells][3]: the estimator's derivative bounds by
 * relative cell (x fastest) and direction, NaN for nearby cells; relative_cell [n]; velocity [n][3]; active_charge
 * [n]; target_charges [n][units]; potential_change [n] (random.expovariate(beta)).  rate [n]: the stored bounding
 * event rate; time [n]: the time displacement (inf for a rate <= 0).  status [n]: _ASSERTION for a nearby cell,
 * target charges that do not sum to 0.0 or a velocity off one positive axis, _INDEX for a cell outside the table. */
int jfgpu_composite_cell_bound_time(const double *upper, const double *lower, int64_t cells,
                                    const int32_t *relative_cell, const double *velocity, const double *active_charge,
                                    const double *target_charges, int32_t units, double dipole_charge,
                                    const double *potential_change, int64_t n, double *rate, double *time,
                                    int32_t *status, void *stream);
/* The cell-veto event time of n events for the sampled relative cells: rate [n] = bound * |active charge| (upper
 * bounds for a positive charge, else lower), time [n] = potential_change / (Walker total * |active charge| * speed).
 * walker_upper / walker_lower [3]: the Walker tables' total rates by direction; the other arguments as for
 * jfgpu_composite_cell_bound_time. */
int jfgpu_composite_cell_veto_time(const double *upper, const double *lower, int64_t cells,
                                   const double *walker_upper, const double *walker_lower,
                                   const int32_t *relative_cell, const double *velocity, const double *active_charge,
                                   const double *potential_change, int64_t n, double *rate, double *time,
                                   int32_t *status, void *stream);

/* Walker's alias table (event_handler/walker.py:53-122), which samples the cell veto's relative cell.
 * jfgpu_walker_table builds it on the HOST from n items in the handler's order (items and rates host arrays; the
 * cell veto gives every non-nearby relative cell with max(bound, 0.0), cell_veto_event_handler.py:148-160):
 * first_item / first_rate / second_item [n] (second_item -1 for an entry of one item), the total and mean rate;
 * JFGPU_ERROR_TABLE where the reference's assertions fail.  jfgpu_walker_sample picks n items on the device from
 * such a table (device arrays): choice [n] the table index of random.choice, draws [n] random.uniform(0.0, mean
 * rate) as values (JFGPU_DRAW_VALUE) or unit draws (JFGPU_DRAW_UNIT); items [n], status [n] (_INDEX for an index
 * outside the table). */
int jfgpu_walker_table(const int32_t *items, const double *rates, int64_t n, int32_t *first_item, double *first_rate,
                       int32_t *second_item, double *total_rate, double *mean_rate);
int jfgpu_walker_sample(const int32_t *first_item, const double *first_rate, const int32_t *second_item, int64_t size,
                        double mean_rate, const int64_t *choice, const double *draws, int32_t draw_mode, int64_t n,
                        int32_t *items, int32_t *status, void *stream);

/* ======================================================================================================
 * Chains: thousands of independent ECMC chains advanced by one kernel with the event loop on the device.
 * ==================================================================================================== */
typedef struct {
    int32_t potential;            /* JFGPU_POT_* */
    int32_t far;                  /* JFGPU_FAR_* */
    int32_t n;                    /* particles of the chain */
    int32_t cells_per_side;
    int32_t neighbor_layers;
    int32_t max_occupants;        /* maximum occupants per cell (1 for the far fields) */
    int32_t initial_active;
    int32_t initial_direction;
    int32_t fourier_cutoff;       /* merged-image Coulomb */
    int32_t position_cutoff;
    int32_t estimator_points;     /* InnerPointEstimator.points_per_side */
    int32_t reserved;
    double system_length;
    double beta;
    double chain_time;
    double speed;
    double hs_radius;             /* hard sphere radius / hard-core radius of a Coulomb system (0 = none) */
    double lj_prefactor;
    double lj_sigma;
    double coulomb_prefactor;
    double bound_prefactor;       /* inverse-power Coulomb bounding prefactor */
    double ewald_alpha;
    double estimator_prefactor;
    uint64_t rng_key;             /* key of the chain's keyed random numbers */
} JfgpuChainDesc;

/* per-chain lifting state (device array of n_chains) */
typedef struct {
    double time_q, time_r;        /* time stamp of the active unit (quotient and remainder of t / 1) */
    double eoc_q, eoc_r;          /* candidate time of the end-of-chain event */
    int64_t events;               /* committed events */
    int64_t bound_warnings;       /* thinning events with a real rate above the bounding rate */
    int64_t refine_fallbacks;     /* mixed mode: events re-solved entirely in FP64 */
    int64_t candidates;           /* pair candidates solved (nearby occupants and surplus units) */
    int64_t refined;              /* mixed mode: candidates re-solved in FP64 */
    int32_t active;
    int32_t direction;
    int32_t eoc_new_active;
    int32_t occ_active;           /* identifier the occupancy treats as active (-1 = none) */
    int32_t occ_cell;             /* active cell of the occupancy */
    int32_t n_surplus;
    int32_t status;               /* JFGPU_STATUS_* of the first failure; the chain stops */
    int32_t stopped;              /* the chain reached the stop time of the current call */
    double lift_sum;              /* sum over the accepted liftings of the separation target - active along the
                                     direction of motion (the excess displacement of the chains, whose ratio to the
                                     total displacement gives the pressure: beta P / rho = 1 + lift_sum / (v t)) */
    int64_t liftings;             /* accepted liftings (pair, bounded, cell-bounding and cell-veto events) */
    int64_t far_lookups;          /* mixed mode, cell-bounding far field: units whose keyed draw passed the rejection
                                     by the largest far rate, whose role word the screen then read */
} JfgpuChainState;

/* one committed event (device log array [n_chains][log_capacity]) */
typedef struct {
    int32_t kind, moved, target, new_active, new_direction, accepted;
    double time_q, time_r;
    double x, y, z;
} JfgpuEvent;

/* ======================================================================================================
 * Flexible water: batched chains of `molecules` water molecules (hydrogen, oxygen, hydrogen; unit 3 m + t of
 * molecule m) with harmonic O-H and H-H bonds (DisplacedEvenPowerPotential, power 2), Lennard-Jones between the
 * oxygens and one Coulomb factor per pair of molecules (the composite-object event above, inside-first,
 * outside-first or ratio lifting), for every pair of molecules, and the periodic-direction end of chain.  One
 * block advances one chain, in FP64 with the reference's arithmetic.  Replaces the reference's event loop
 * (mediator/single_process_mediator.py:91-156) over the handlers of these factors:
 * two_leaf_unit_event_handler.py:98-154, two_composite_object_summed_bounding_potential_event_handler.py:119-202,
 * single_independent_active_periodic_direction_end_of_chain_event_handler.py:151-237.
 * ==================================================================================================== */
typedef struct {
    int32_t molecules;            /* per chain, 2..4096 */
    int32_t lifting;              /* JFGPU_LIFTING_* */
    int32_t fourier_cutoff;       /* merged-image Coulomb */
    int32_t position_cutoff;
    int32_t initial_active;       /* unit index */
    int32_t initial_direction;
    int32_t mode;                 /* JFGPU_MODE_EXACT: every candidate and merged-image sum in FP64;
                                     JFGPU_MODE_MIXED: the Coulomb candidates are screened in FP32 with error bounds
                                     and only those that may come first are solved in FP64, and the thinning of a
                                     Coulomb event rejects on FP32 sums with an error bound when the bound decides,
                                     else takes the FP64 sums (the same outcomes as the exact mode) */
    int32_t reserved;
    double system_length;
    double beta;
    double chain_time;
    double speed;
    double oh_r0, oh_prefactor;   /* O-H bond: prefactor (r - r0)^2 */
    double hh_r0, hh_prefactor;   /* H-H bond */
    double lj_prefactor, lj_sigma;
    double coulomb_prefactor, bound_prefactor, alpha;
    uint64_t seed;                /* chain c draws its random numbers with the key of (seed, c) */
} JfgpuWaterDesc;

/* per-chain state of a water batch (device array [chains]) */
typedef struct {
    double time_q, time_r;        /* time stamp of the active unit */
    double eoc_q, eoc_r;          /* end-of-chain candidate */
    int32_t active, direction, eoc_new_active, status;
    int32_t stopped;              /* the chain reached the stop time of the current call */
    int32_t reserved;
    int64_t events;               /* committed events: the event index of the keyed draws */
    int64_t composite_events, composite_accepted, bond_events, lj_events, eoc_events;
    int64_t thinning_exact;       /* Coulomb events whose thinning took the FP64 sums (all of them in exact mode) */
    int64_t refined_items;        /* candidate items solved in FP64 (every item in exact mode) */
} JfgpuWaterState;

/* the model on the current device (the Fourier table of the Coulomb factor) */
int jfgpu_water_create(const JfgpuWaterDesc *desc, void **water);
void jfgpu_water_destroy(void *water);
/* chains first_chain .. first_chain + chains - 1 at time 0: the initial active unit and direction, the first end
 * of chain (time chain_time, new active unit drawn for event 0) */
int jfgpu_water_init(void *water, JfgpuWaterState *state, int64_t chains, int64_t first_chain, void *stream);
/* up to `events` events of every chain, stopping at the stop time (stop_q, stop_r as Time quotient and remainder;
 * inf, inf for none): a chain whose next event would come at or after it (the stop wins ties) has its active unit
 * time-sliced to the stop time, `stopped` set and no further event in this call, like the reference's end of run.
 * positions [chains][3 molecules][3] and charges [3 molecules] are device arrays; log [chains][events] (may be
 * null) receives every committed event.  One block of warps_per_block warps runs one chain, 1..8 (0: 3). */
int jfgpu_water_run(void *water, double *positions, const double *charges, JfgpuWaterState *state, int64_t chains,
                    int64_t first_chain, int64_t events, double stop_q, double stop_r, JfgpuEvent *log,
                    int32_t warps_per_block, void *stream);

/* Water with molecular cells.  Replaces the reference's SingleProcessMediator loop over its water cell-veto
 * configuration (config_files/2018_JCP_149_064113/water/coulomb_cell_veto_lj_inverted.ini): the molecules' root
 * units (barycentres) in SingleActiveCellOccupancy (activator/internal_state/single_active_cell_occupancy.py:95-203,
 * cell_level 1, one occupant per cell), the summed-bounding Coulomb factor with the molecules of the nearby cells
 * (ExcludedCellsTagger, activator/tagger/excluded_cells_tagger.py:107-132) and with the surplus molecules
 * (SurplusCellsTagger, surplus_cells_tagger.py:107-131), the molecular cell veto
 * (CompositeObjectCellVetoEventHandler, event_handler/composite_object_cell_veto_event_handler.py:110-162) and the
 * cell-boundary event of the active root unit (CellBoundaryEventHandler, event_handler/cell_boundary_event_handler.py:
 * 98-173), which keeps the bond and Lennard-Jones candidates alive. */
typedef struct {
    double pair_q, pair_r;        /* earliest bond / Lennard-Jones candidate (inf: none), kept across cell boundaries */
    double snap_leaf[3], snap_root[3];  /* the active leaf and root unit as that candidate's in-state holds them */
    double snap_q, snap_r;        /* ... at this time stamp */
    int32_t pair_kind, pair_target;
    int32_t pairs_valid;          /* the candidate above is alive (created, then only cell-boundary events) */
    int32_t occ_active, occ_cell; /* the occupancy's active molecule (-1: none) and its cell */
    int32_t reserved;
    int64_t boundary_events;
    int64_t veto_events, veto_targets;  /* far-field events (cell veto or cell bounding) and those with a target */
} JfgpuWaterCellState;

typedef struct {
    double *roots;                /* [chains][molecules][3] root positions */
    int32_t *occupancy;           /* [chains][cells]: the occupant molecule, -1 when empty */
    int32_t *surplus;             /* [chains][molecules]: the cell of a surplus molecule, -1 otherwise */
    JfgpuWaterCellState *cell_state;  /* [chains] */
    double *root_log;             /* [chains][events][3] root of the moved unit's molecule after every event (may be
                                     null) */
} JfgpuWaterCellBuffers;

/* attach the cell system to a water model: cells_per_side^3 cuboid periodic cells with neighbor_layers layers of
 * nearby cells, and the molecular cell veto's bound tables (host arrays [cells][3]: the upper and the negated lower
 * derivative bound of every relative cell and direction, as the estimator filled
 * CellVetoEventHandler._derivative_bounds, abstracts/cell_veto_event_handler.py:134-160; NaN for the nearby cells),
 * from which the Walker tables are built in the reference's order.  cells_per_side 1..32.  keep_pairs: the cell
 * boundary's tagger trashes only the cell-based factors, so the bond and Lennard-Jones candidates outlive it (the
 * reference's water cell-veto configuration); 0: it trashes them too.  far: JFGPU_FAR_CELL_VETO (the molecular cell
 * veto) or JFGPU_FAR_CELL_BOUNDING (CellBoundingPotentialTagger with TwoCompositeObjectCellBoundingPotentialEventHandler,
 * two_composite_object_cell_bounding_potential_event_handler.py:153-265: a factor for every occupied far cell, the
 * charge factor over dipole_charge as DipoleMonteCarloEstimator.charge_correction_factor forms it). */
int jfgpu_water_set_cells(void *water, int32_t cells_per_side, int32_t neighbor_layers, const double *bounds_upper,
                          const double *bounds_lower, int32_t keep_pairs, int32_t far, double dipole_charge);
/* the occupancy of chains first .. first + chains - 1 from their roots (root nodes in order, the first molecule of a
 * cell its occupant, the others surplus) and a fresh cell state; with jfgpu_water_init for the rest of the state */
int jfgpu_water_cells_init(void *water, const JfgpuWaterCellBuffers *buffers, int64_t chains, void *stream);
/* jfgpu_water_run with the molecular cells (arguments as there) */
int jfgpu_water_cells_run(void *water, double *positions, const double *charges, JfgpuWaterState *state,
                          const JfgpuWaterCellBuffers *buffers, int64_t chains, int64_t first_chain, int64_t events,
                          double stop_q, double stop_r, JfgpuEvent *log, int32_t warps_per_block, void *stream);

/* device buffers of a chain batch, all owned by the caller; sizes from jfgpu_engine_layout */
typedef struct {
    double *positions;            /* [particles][3], chain c at particle_offset[c] */
    float *positions32;           /* [particles][4]: FP32 mirror (x, y, z, charge) of the mixed mode */
    double *charges;              /* [particles] (may be NULL for uncharged systems) */
    int32_t *occupancy;           /* [occupancy_slots] */
    int32_t *surplus;             /* [particles] */
    int32_t *roles;               /* [particles]: cell axes (x | y << 8 | z << 16) of every unit's occupancy entry;
                                     for surplus units bit 24 and the unit's index in the surplus list instead;
                                     bit 25 for the occupancy's active unit */
    JfgpuChainState *state;       /* [n_chains] */
    float *cell_slots;            /* [occupancy_slots][4]: cell-ordered FP32 mirror of the occupancy, the occupant's
                                     (x, y, z) and its identifier's bits as the fourth float (bits -1 when empty);
                                     kept by the engine, rebuilt by jfgpu_chains_refresh_mirror */
} JfgpuBuffers;

typedef struct {
    int64_t n_chains;
    int64_t particles;            /* sum of n over chains */
    int64_t occupancy_slots;      /* sum of cells * max_occupants over chains */
    int64_t table_bytes;          /* device bytes of the engine's own tables */
} JfgpuLayout;

typedef struct JfgpuEngine JfgpuEngine;

/* Build an engine for n_chains chains: geometry tables, far-field bound tables (estimator scan on the GPU)
 * and Walker tables.  Chains with equal far-field parameters share tables.  Returns JFGPU_OK and *engine. */
int jfgpu_engine_create(const JfgpuChainDesc *chains, int64_t n_chains, void *stream, JfgpuEngine **engine);
void jfgpu_engine_destroy(JfgpuEngine *engine);
int jfgpu_engine_layout(const JfgpuEngine *engine, JfgpuLayout *layout);
/* host arrays [n_chains]: first particle and first occupancy slot of every chain */
int jfgpu_engine_offsets(const JfgpuEngine *engine, int64_t *particle_offset, int64_t *occupancy_offset);
/* host copy of the far-field tables of a chain: upper [cells][3], lower [cells][3] (negated lower bound) */
int jfgpu_engine_bounds(const JfgpuEngine *engine, int64_t chain, double *upper, double *lower, int64_t capacity);

/* Start the chains from buffers->positions (and charges): FP32 mirror, cell occupancy, surplus lists, lifting
 * state at time 0 with the first end-of-chain candidate (InitialChainStartOfRunEventHandler). */
int jfgpu_chains_init(JfgpuEngine *engine, const JfgpuBuffers *buffers, void *stream);

/* Advance chains [first_chain, first_chain + count) by at most max_events committed events each, or until the
 * next event time reaches the stop time (stop_q = +inf: none), where the active unit is time-sliced to the
 * stop time.  mode = JFGPU_MODE_*.  log (device, may be NULL) receives [count][log_capacity] events. */
int jfgpu_chains_run(JfgpuEngine *engine, const JfgpuBuffers *buffers, int64_t first_chain, int64_t count,
                     int64_t max_events, double stop_q, double stop_r, int32_t mode, JfgpuEvent *log,
                     int64_t log_capacity, void *stream);

/* Autotuned launch shape of the mixed mode: warps per block used by jfgpu_chains_run (1..8). */
int jfgpu_chains_set_block_warps(JfgpuEngine *engine, int32_t warps_per_block);

/* Mixed mode: an event whose refine list (the FP32 near-winners and flagged candidates) holds more than `limit`
 * entries is re-solved entirely in FP64 (counted in refine_fallbacks).  1..JFGPU_REFINE_LIST_MAX, default the
 * maximum; every limit gives the same events, times and positions. */
#define JFGPU_REFINE_LIST_MAX 28
int jfgpu_chains_set_refine_limit(JfgpuEngine *engine, int32_t limit);

/* Rewrite the FP32 mirrors of chains [first_chain, first_chain + count): buffers->positions32 (x, y, z, charge) from
 * their FP64 positions (and charges), then buffers->cell_slots from the occupancy and that mirror.  For hosts that
 * upload positions and occupancy between runs, instead of uploading the mirrors as well.  The mirrors are otherwise
 * kept by the engine (jfgpu_chains_init and every committed event). */
int jfgpu_chains_refresh_mirror(JfgpuEngine *engine, const JfgpuBuffers *buffers, int64_t first_chain, int64_t count,
                                void *stream);

/* Observables of chains [first_chain, first_chain + count) at their current positions, for the estimators of
 * long runs (all pairs of a chain, minimum-image separations from the FP32 mirror):
 *   energy    [count] (device, may be NULL): potential energy of the chain's pair potential, the sum over pairs
 *             of the Lennard-Jones potential (lennard_jones_potential.py:83-98), 0 for hard spheres, NaN for
 *             merged-image Coulomb chains (the reference defines no Coulomb energy);
 *   histogram [count][bins] (device, may be NULL): pair distances in [0, r_max) with bins equal bins, ADDED to
 *             the array (samples accumulate over calls); 1 <= bins <= 4096.
 * The pair-separation samples of separation_output_handler.py:75-97, reduced on the device. */
int jfgpu_chains_observe(JfgpuEngine *engine, const JfgpuBuffers *buffers, int64_t first_chain, int64_t count,
                         int32_t bins, double r_max, double *energy, uint64_t *histogram, void *stream);

/* Chain groups of the mixed mode: the chains of one jfgpu_chains_run call are split into `groups` contiguous
 * groups (1..8) whose event rounds run on streams of their own, forked from and joined back into the caller's
 * stream, so that one group's FP64 re-solves overlap another group's FP32 screening.  Default 1. */
int jfgpu_chains_set_groups(JfgpuEngine *engine, int32_t groups);

/* CUDA graphs for the event rounds of the mixed mode (default on): the launches of a run call are captured once per
 * shape (chains, rounds, stop time, buffers, launch shape) and replayed as one graph launch afterwards; calls with
 * an event log, or on a stream the caller is capturing, launch plainly.  Results are identical either way. */
int jfgpu_chains_set_graphs(JfgpuEngine *engine, int32_t enable);

/* Kernel launches issued by the library since the engine was created (all kernels of this library). */
int64_t jfgpu_engine_launch_count(const JfgpuEngine *engine);

/* kernel kinds of jfgpu_engine_kernel_times */
#define JFGPU_KERNEL_SCREEN 0          /* FP32 screening of every candidate (one warp per chain) */
#define JFGPU_KERNEL_REFINE 1          /* not launched: the settle kernel runs the FP64 re-solves */
#define JFGPU_KERNEL_RESOLVE 2         /* the settle kernel: FP64 re-solves of the listed near-winners, single
                                          candidates, argmin, commit and occupancy update */
#define JFGPU_KERNEL_CHAINS 3          /* the FP64 event loop of JFGPU_MODE_EXACT */
#define JFGPU_KERNEL_INIT 4            /* chain start */
#define JFGPU_KERNEL_OBSERVE 5         /* observables of jfgpu_chains_observe */
#define JFGPU_KERNEL_KINDS 6

/* Per-kernel device time.  While timing is on (enable = k >= 1), the chain launches of jfgpu_chains_init,
 * jfgpu_chains_run and jfgpu_chains_observe are bracketed by CUDA events on the stream they are launched on; in
 * the mixed mode only every k-th event round is bracketed (k = 1: all), so that the events barely perturb the
 * run they measure.  enable = 0 switches timing off.  jfgpu_engine_kernel_times waits for those events and
 * returns, per kernel kind, the milliseconds and the timed launches accumulated since the last reset (arrays of
 * JFGPU_KERNEL_KINDS entries; reset != 0 clears the totals after reading). */
int jfgpu_engine_set_timing(JfgpuEngine *engine, int32_t enable);
int jfgpu_engine_kernel_times(JfgpuEngine *engine, double *milliseconds, int64_t *launches, int32_t reset);

/* ======================================================================================================
 * Initial states (host): random sequential addition of n hard spheres of the given radius in the periodic cube of
 * side system_length, the trial points drawn from a SplitMix64 stream of `seed`; a trial closer than one diameter to
 * a placed sphere (minimum image) is rejected.  positions [n][3] (host) receive the spheres in placement order.
 * JFGPU_ERROR_TABLE after max_trials trials without n spheres.  The reference places atoms without overlap rejection
 * (input_output_handler/input_handler/random_node_creator/atom_random_node_creator.py:56-67); its hard-sphere runs need
 * non-overlapping starts, which this supplies for the batched hard-sphere workloads.
 * ==================================================================================================== */
int jfgpu_random_sequential_addition(int64_t n, double radius, double system_length, uint64_t seed,
                                     int64_t max_trials, double *positions);

const char *jfgpu_error_string(int code);
int jfgpu_version(void);

#ifdef __cplusplus
}
#endif
#endif
