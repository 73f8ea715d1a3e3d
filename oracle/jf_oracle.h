/*
 * jf_oracle.h -- CPU restatement of JeLLyFysh's event-time path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU product is tested against: it is
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.
 * The product (jellyfysh_gb300) never links, loads or calls it.
 *
 * Every function restates the reference's arithmetic with CPython 3.12 float semantics
 * (IEEE double, no FMA contraction, `sum()` with Neumaier compensation, `%` and
 * `divmod` with the sign of the divisor), citing the reference file:line it follows.
 */
#ifndef JF_ORACLE_H
#define JF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirror the exceptions the reference would raise) ---- */
#define JFO_OK 0
#define JFO_VALUE_ERROR 1      /* math.sqrt of a negative number (ValueError) */
#define JFO_ASSERT 2           /* a failed `assert` in the reference */
#define JFO_ZERO_DIVISION 3    /* ZeroDivisionError of a Python float division */
#define JFO_COMPLEX 4          /* negative ** fractional (Python returns complex, then crashes) */
#define JFO_BAD_CONFIG 5
#define JFO_ALLOC 6
#define JFO_CELL_RANGE 7       /* position_to_cell index outside the cell list (IndexError) */
#define JFO_LIFTING 9          /* LiftingSchemeError: no active unit in the lifting table */
#define JFO_INDEX 10           /* IndexError: no negative derivative in the lifting table */

/* ---- event kinds recorded in the event log ---- */
#define JFO_EV_PAIR 0          /* inverted pair potential (hard sphere / Lennard-Jones): lifting */
#define JFO_EV_BOUNDED 1       /* bounding-potential pair event, thinning with the real derivative */
#define JFO_EV_HARDCORE 2      /* hard-core pair event of a Coulomb system: lifting */
#define JFO_EV_CELL_BOUNDING 3 /* far-field cell-bounding-potential event (thinning) */
#define JFO_EV_CELL_VETO 4     /* far-field cell-veto event (thinning) */
#define JFO_EV_BOUNDARY 5      /* cell-boundary event */
#define JFO_EV_END_OF_CHAIN 6  /* end-of-chain event */
#define JFO_EV_STOP 7          /* run stopped at a stop time (sampling / end-of-run time slice) */
#define JFO_EV_BOND 8          /* intramolecular bond (displaced even power) of a water molecule: lifting */
#define JFO_EV_COMPOSITE 9     /* Coulomb factor of two molecules: thinning and lifting within both */

/* ---- pair potential kinds of a chain system ---- */
#define JFO_POT_HARD_SPHERE 0
#define JFO_POT_LENNARD_JONES 1
#define JFO_POT_COULOMB 2      /* merged-image Coulomb, bounded by the inverse-power Coulomb bound */

/* ---- far-field kinds ---- */
#define JFO_FAR_NONE 0
#define JFO_FAR_CELL_VETO 1
#define JFO_FAR_CELL_BOUNDING 2

/* ---- random-number kinds (keyed draws) ---- */
#define JFO_RNG_PAIR 0         /* potential change of the pair handler of a target */
#define JFO_RNG_THIN 1         /* uniform of a thinning decision */
#define JFO_RNG_VETO_TIME 2    /* potential change of the cell-veto handler */
#define JFO_RNG_VETO_CHOICE 3  /* Walker table entry */
#define JFO_RNG_VETO_UNIFORM 4 /* Walker uniform */
#define JFO_RNG_NEW_ACTIVE 5   /* end-of-chain randint (target 0: molecule or atom, 1: unit of the molecule) */
#define JFO_RNG_COMPOSITE 6    /* potential change of a Coulomb factor of two molecules, per target unit */
#define JFO_RNG_LIFT 7         /* uniform of the lifting scheme */
#define JFO_RNG_CELL_BOUND 8   /* potential change of a molecular cell-bounding factor, by target molecule */

/* primitives */
double jfo_py_mod(double x, double y);
void jfo_py_divmod(double x, double y, double *quotient, double *remainder);
double jfo_py_sum3(double a, double b, double c);
double jfo_py_sum(const double *values, int n);
void jfo_time_add(double q, double r, double dt, double *out_q, double *out_r);
double jfo_time_sub(double q1, double r1, double q2, double r2);
int jfo_time_lt(double q1, double r1, double q2, double r2);

/* keyed random numbers */
uint64_t jfo_chain_key(uint64_t seed, uint64_t chain);
uint64_t jfo_draw(uint64_t key, uint64_t event, uint32_t kind, uint32_t target);
double jfo_uniform(uint64_t bits);
double jfo_log(double x);
double jfo_expovariate(uint64_t bits, double beta);
uint32_t jfo_randbelow(uint64_t bits, uint32_t n);

/* potentials (velocity given as 3 components, separation mutable copy is made inside) */
int jfo_hs_displacement(double radius, const double *velocity, const double *separation, double *out);
int jfo_ip_displacement(double power, double prefactor, const double *velocity, const double *separation,
                        double charge_one, double charge_two, double potential_change, double *out);
int jfo_ip_derivative(double power, double prefactor, const double *velocity, const double *separation,
                      double charge_one, double charge_two, double *out);
int jfo_lj_displacement(double prefactor, double sigma, const double *velocity, const double *separation,
                        double potential_change, double *out);
int jfo_lj_derivative(double prefactor, double sigma, const double *velocity, const double *separation,
                      double *out);
int jfo_dep_displacement(double r0, int power, double prefactor, const double *velocity,
                         const double *separation, double potential_change, double *out);
int jfo_dep_derivative(double r0, int power, double prefactor, const double *velocity,
                       const double *separation, double *out);
int jfo_ipcb_displacement(double prefactor, double system_length, const double *velocity,
                          const double *separation, double charge_one, double charge_two,
                          double potential_change, double *out);
int jfo_ipcb_derivative(double prefactor, const double *velocity, const double *separation,
                        double charge_one, double charge_two, double *out);
/* merged-image Coulomb: x-derivative of the Ewald sum (no prefactor, unit charges) */
double jfo_mic_x_derivative(double alpha, int fourier_cutoff, int position_cutoff, double system_length,
                            double sx, double sy, double sz);
int jfo_mic_derivative(double alpha, int fourier_cutoff, int position_cutoff, double prefactor,
                       double system_length, const double *velocity, const double *separation,
                       double charge_one, double charge_two, double *out);

/* lifting schemes of composite objects (lifting/lifting.py:47-108 with inside_first_lifting.py:37-54,
 * outside_first_lifting.py:38-55, ratio_lifting.py:38-56).  scheme 0 inside-first, 1 outside-first, 2 ratio;
 * unit_draw 0: draw is the value random.uniform returned, 1: draw is random() and the value is formed as
 * random.uniform does.  *selected = table index of the new active unit, *bound = b of the deciding
 * random.uniform(0.0, b) call (NaN if the reference raises first). */
int jfo_lifting(int scheme, int unit_draw, const double *rates, const int32_t *active, int count, double draw,
                int64_t *selected, double *bound);

/* events between two composite objects of `units` point charges each
 * (two_composite_object_summed_bounding_potential_event_handler.py:119-202): merged-image Coulomb
 * (alpha, fourier_cutoff, position_cutoff, coulomb_prefactor) bounded by the inverse-power Coulomb bound
 * (bound_prefactor).  Positions are [units][3]; scheme and unit_draw as for jfo_lifting. */
int jfo_composite_event_time(int units, double alpha, int fourier_cutoff, int position_cutoff,
                             double coulomb_prefactor, double bound_prefactor, double system_length,
                             const double *velocity, const double *active_position, double active_charge,
                             const double *target_positions, const double *target_charges,
                             const double *potential_changes, double *displacement);
int jfo_composite_out_state(int units, int scheme, int unit_draw, double alpha, int fourier_cutoff,
                            int position_cutoff, double coulomb_prefactor, double bound_prefactor,
                            double system_length, const double *velocity, const double *local_positions,
                            const double *local_charges, int active_index, const double *target_positions,
                            const double *target_charges, int local_first, const double *draws, int *new_active,
                            double *bounding_rate, double *event_rate);
/* the molecular cell-bounding and cell-veto handlers: the out-state against a given bounding event rate, the event
 * times from the bound of the relative cell */
int jfo_composite_bounded_out_state(int units, int scheme, int unit_draw, double alpha, int fourier_cutoff,
                                    int position_cutoff, double coulomb_prefactor, double system_length,
                                    const double *velocity, const double *local_positions,
                                    const double *local_charges, int active_index, const double *target_positions,
                                    const double *target_charges, int local_first, double bounding_rate,
                                    const double *draws, int *new_active, double *event_rate);
int jfo_composite_cell_bound_time(const double *upper, const double *lower, const double *velocity,
                                  double active_charge,
                                  const double *target_charges, int units, double dipole_charge,
                                  double potential_change, double *rate, double *time);
int jfo_composite_cell_veto_time(const double *upper, const double *lower, const double *walker_upper,
                                 const double *walker_lower, const double *velocity, double active_charge,
                                 double potential_change, double *rate, double *time);

/* Walker's alias table (event_handler/walker.py:53-122) */
int jfo_walker_table(const int *items, const double *rates, int n, int *first_item, double *first_rate,
                     int *second_item, double *total_rate, double *mean_rate);
int jfo_walker_pick(const int *first_item, const double *first_rate, const int *second_item, int size, int choice,
                    double uniform);

/* cells */
void jfo_cell_bounds(double system_length, int cells_per_side, double *cell_min, double *cell_max);

/* chain system description */
typedef struct {
    int n;                  /* number of particles */
    double system_length;   /* cubic box side */
    int cells_per_side;
    int neighbor_layers;
    int max_occupants;      /* maximum occupants per cell (>= 1) */
    double beta;
    double chain_time;
    double speed;
    int initial_direction;
    int initial_active;
    int potential;          /* JFO_POT_* */
    double hs_radius;       /* hard-sphere radius (potential 0) or hard-core radius (potential 2, 0 = none) */
    double lj_prefactor;
    double lj_sigma;
    double coulomb_prefactor;
    double bound_prefactor; /* inverse-power Coulomb bounding prefactor */
    double ewald_alpha;
    int fourier_cutoff;
    int position_cutoff;
    int far;                /* JFO_FAR_* */
    int estimator_points;   /* InnerPointEstimator points_per_side */
    double estimator_prefactor;
    uint64_t rng_key;
} JfoSystem;

/* one committed event */
typedef struct {
    int32_t kind;
    int32_t moved;          /* the particle that was active during the event */
    int32_t target;         /* pair target / looked-up occupant, -1 if none */
    int32_t new_active;
    int32_t new_direction;
    int32_t accepted;       /* thinning outcome (1 for events without thinning that lift) */
    double time_q, time_r;  /* event time */
    double x, y, z;         /* committed position of the moved particle */
} JfoEvent;

/* flexible water: molecules of three units (hydrogen, oxygen, hydrogen; unit 3 m + t), harmonic O-H and H-H bonds
 * (displaced even power, power 2), Lennard-Jones between oxygens and a Coulomb factor of every pair of molecules
 * (merged-image Coulomb bounded by the summed inverse-power Coulomb bound, lifting scheme `lifting`), all pairs of
 * molecules, periodic-direction end of chain */
typedef struct {
    int molecules;
    double system_length;
    double beta;
    double chain_time;
    double speed;
    int initial_direction;
    int initial_active;     /* unit index */
    double oh_r0, oh_prefactor;
    double hh_r0, hh_prefactor;
    double lj_prefactor, lj_sigma;
    double coulomb_prefactor, bound_prefactor, ewald_alpha;
    int fourier_cutoff, position_cutoff;
    int lifting;            /* 0 inside-first, 1 outside-first, 2 ratio */
    uint64_t rng_key;
} JfoWaterSystem;

typedef struct JfoWater JfoWater;
JfoWater *jfo_water_create(const JfoWaterSystem *system, const double *positions, const double *charges, int *status);
void jfo_water_destroy(JfoWater *water);
/* runs up to max_events events; returns the number run; *status is JFO_OK or the first failure */
int64_t jfo_water_run(JfoWater *water, int64_t max_events, JfoEvent *log, int *status);
/* the same with the root position of the moved unit's molecule after every event (root_log [max_events][3], may be
 * NULL; molecular cells only) */
int64_t jfo_water_run_roots(JfoWater *water, int64_t max_events, JfoEvent *log, double *root_log, int *status);
/* flexible water with molecular cells of root units (cells_per_side^3 cuboid periodic cells, neighbor_layers): the
 * Coulomb factor with the molecules of the nearby cells and the surplus molecules, the far field (far
 * JFO_FAR_CELL_VETO: the molecular cell veto; JFO_FAR_CELL_BOUNDING: the molecular cell-bounding factor of every
 * occupied far cell, charge factor over dipole_charge) with the given bound tables ([cells][3] upper and negated lower
 * bounds, NaN for the nearby cells) and the cell-boundary events of the active root unit; roots [molecules][3] are
 * the initial root positions; keep_pairs: the bond and Lennard-Jones candidates outlive a cell boundary (its tagger
 * trashes only the cell-based factors) */
JfoWater *jfo_water_cells_create(const JfoWaterSystem *system, int cells_per_side, int neighbor_layers,
                                 const double *positions, const double *charges, const double *roots,
                                 const double *bounds_upper, const double *bounds_lower, int keep_pairs, int far,
                                 double dipole_charge, int *status);
void jfo_water_roots(const JfoWater *water, double *roots);
void jfo_water_positions(const JfoWater *water, double *positions);
void jfo_water_state(const JfoWater *water, int64_t *event_count, int *active, int *direction, double *time_q,
                     double *time_r);

typedef struct JfoChain JfoChain;

JfoChain *jfo_chain_create(const JfoSystem *system, const double *positions, const double *charges, int *status);
void jfo_chain_destroy(JfoChain *chain);
/* Run until max_events events are committed or the next event time exceeds the stop time
 * (stop_q = inf: no stop).  Returns the number of committed events; log may be NULL. */
int64_t jfo_chain_run(JfoChain *chain, int64_t max_events, double stop_q, double stop_r, JfoEvent *log,
                      int *status);
void jfo_chain_positions(const JfoChain *chain, double *positions);
void jfo_chain_state(const JfoChain *chain, int64_t *event_count, int *active, int *direction,
                     double *time_q, double *time_r);
int jfo_chain_occupancy(const JfoChain *chain, int32_t *owner);
/* sum over the accepted liftings of the separation target - active along the direction of motion, and their
 * number (the harness's pressure estimator: beta P / rho = 1 + lift_sum / (speed * elapsed time)) */
void jfo_chain_liftings(const JfoChain *chain, double *lift_sum, int64_t *liftings);
int jfo_chain_bounds(const JfoChain *chain, double *bounds, int capacity);
int jfo_chain_walker(const JfoChain *chain, int direction, int which, int32_t *cells, double *rates, int capacity,
                     double *total_rate);

#ifdef __cplusplus
}
#endif
#endif
